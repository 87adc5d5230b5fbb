// Batched gradient of the THERMAL z-march with fixed temperature fields (host driver and
// the shg_thgrad_* C ABI).
//
// Each solve's temperature field comes from Solver::run (-DTHERMAL, Solver.h:287-340) run
// once on the device, or is given. From it the solve keeps per-voxel coupling tables
// (Solver.h:44-63 with PhaseMatching.h:12-54), its propagators and Gaussian pump at the
// centre temperature T[NX/2, NY/2, 0] (Efields.h:77,110). The forward pass is the thermal
// CWES (Solver.h:245-276) without heat-source updates, run for all solves at once; the
// loss of solve b is its SH power at the top of slice NZ-1, the gradient is with respect
// to its input pump (Wirtinger form dL/dRe + i dL/dIm). The whole pass, batched over
// solves, is captured once in a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <vector>

#include "../../include/shg.h"
#include "shg_adjoint.h"
#include "shg_adjoint_th.h"
#include "shg_thermal_host.h"

namespace shg {

#define TG_CUDA(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            set_error(std::string("thgrad: ") + #call + ": " + cudaGetErrorString(e_));               \
            return e_ == cudaErrorMemoryAllocation ? SHG_ERR_NOMEM : SHG_ERR_CUDA;                     \
        }                                                                                              \
    } while (0)

#define TG_TRY(expr)         \
    do {                     \
        int rc_ = (expr);    \
        if (rc_) return rc_; \
    } while (0)

ThermalGradBatch::~ThermalGradBatch() {
    drop_graphs();
    if (cap_) cudaStreamDestroy(cap_);
    if (side_) cudaStreamDestroy(side_);
    if (ev_) cudaEventDestroy(ev_);
    for (void *p : {(void *)T_, (void *)coef_, (void *)props_, (void *)pump0_, (void *)stepc_, (void *)setup_acc_,
                    (void *)seed_, (void *)d_desc_, work_})
        if (p) cudaFree(p);
}

void ThermalGradBatch::drop_graphs() {
    if (g_fwd_) cudaGraphExecDestroy(g_fwd_);
    if (g_grad_) cudaGraphExecDestroy(g_grad_);
    g_fwd_ = g_grad_ = nullptr;
    g_grad_L_ = -1;
}

int ThermalGradBatch::create(const shg_config &cfg, int count) {
    if (cfg.nx != cfg.ny || !line_length_supported(cfg.nx) || cfg.nz < 2 || count < 1 || count > 16383) {
        set_error("shg_thgrad_create: needs NX = NY a power of two in [16, 256], NZ >= 2, 1 <= count < 16384");
        return SHG_ERR_UNSUPPORTED;
    }
    cfg_ = cfg;
    cfg_.thermal = 1;
    n_ = cfg.nx;
    nz_ = cfg.nz;
    K_ = nz_ - 1;
    count_ = count;
    nn_ = (size_t)n_ * n_;
    tsize_ = nn_ * nz_;
    TG_CUDA(cudaSetDevice(cfg.device));
    TG_TRY(ensure_twiddles(cfg.device));
    const size_t c = (size_t)count;
    TG_TRY(device_fits(c * (tsize_ * sizeof(float) + (size_t)K_ * nn_ * sizeof(float4) + 3 * nn_ * sizeof(float2)),
                       "batched THERMAL gradient"));
    TG_CUDA(cudaMalloc(&T_, c * tsize_ * sizeof(float)));
    TG_CUDA(cudaMalloc(&coef_, c * (size_t)K_ * nn_ * sizeof(float4)));
    TG_CUDA(cudaMalloc(&props_, c * 2 * nn_ * sizeof(float2)));
    TG_CUDA(cudaMalloc(&pump0_, c * nn_ * sizeof(float2)));
    TG_CUDA(cudaMalloc(&stepc_, c * (size_t)nz_ * sizeof(float4)));
    TG_CUDA(cudaMalloc(&setup_acc_, c * 4 * sizeof(double)));
    TG_CUDA(cudaMalloc(&seed_, c * sizeof(double)));
    TG_CUDA(cudaMalloc(&d_desc_, c * sizeof(InstDesc)));
    fixed_bytes_ = c * (tsize_ * sizeof(float) + (size_t)K_ * nn_ * sizeof(float4) + 3 * nn_ * sizeof(float2) +
                        (size_t)nz_ * sizeof(float4) + 5 * sizeof(double) + sizeof(InstDesc));
    h_desc_.assign(c, InstDesc{});
    tc_.assign(c, 0.f);
    ready_.assign(c, 0);
    TG_CUDA(cudaStreamCreateWithFlags(&cap_, cudaStreamNonBlocking));
    return SHG_OK;
}

int ThermalGradBatch::ensure_thermal() {
    if (ts_) return SHG_OK;
    ts_.reset(new ThermalSolve);
    return ts_->create(cfg_);
}

// Solve i from the tables of ts_ (built from its current temperature field).
int ThermalGradBatch::setup_solve(int i, float power, float waist, float focal) {
    cudaStream_t st = ts_->stream();
    const float tc = ts_->center_temperature();
    TG_CUDA(cudaMemcpyAsync(T_ + (size_t)i * tsize_, ts_->T_cur(), tsize_ * sizeof(float), cudaMemcpyDeviceToDevice,
                            st));
    TG_CUDA(launch_th_coef_table(ts_->NP(), ts_->NS(), ts_->DK(), coef_ + (size_t)i * K_ * nn_, (int)nn_, K_,
                                 ts_->therm(), st));
    SolveParams sp{n_, nz_, cfg_.lx, cfg_.ly, power, waist, focal, tc, tc, tc};
    InstDesc h;
    std::memset(&h, 0, sizeof(h));
    fill_scalars(cfg_, sp, h);
    h.P = pump0_ + (size_t)i * nn_;
    h.Hp = props_ + (size_t)i * 2 * nn_;
    h.Hs = h.Hp + nn_;
    h.stepc = stepc_ + (size_t)i * nz_;
    h.acc = setup_acc_ + (size_t)i * 4;
    h.nsteps = K_;
    h.pump_given = 0;
    h_desc_[i] = h;
    tc_[i] = tc;
    TG_CUDA(cudaMemcpyAsync(d_desc_ + i, &h_desc_[i], sizeof(InstDesc), cudaMemcpyHostToDevice, st));
    TG_CUDA(cudaMemsetAsync(h.acc, 0, 4 * sizeof(double), st));
    // Efields.h:74-126: Gaussian pump and shifted propagators at the centre temperature
    TG_CUDA(launch_setup(d_desc_ + i, 1, (int)nn_, nz_, st));
    // loss scale: P_SH = 1/2 eps0 c n_s(tc) dx dy sum |S|^2 (the efficiency's convention)
    const float ns = crystal_index(cfg_.crystal, (float)(0.5 * (double)cfg_.lp), tc);
    const double seed = 2.0 * field_power(1.0, ns, h.dx, h.dy);
    TG_CUDA(cudaMemcpyAsync(seed_ + i, &seed, sizeof(double), cudaMemcpyHostToDevice, st));
    TG_CUDA(cudaStreamSynchronize(st));
    ready_[i] = 1;
    return SHG_OK;
}

int ThermalGradBatch::solve_temperature(int i, float power, float waist, float focal, float temp, float t_inf,
                                        float t1, float t2, int *counts) {
    if (i < 0 || i >= count_) {
        set_error("shg_thgrad_solve_temperature: solve index out of range");
        return SHG_ERR_INVALID;
    }
    TG_TRY(ensure_thermal());
    TG_TRY(ts_->run(power, waist, focal, temp, t_inf, t1, t2));
    if (counts) ts_->counts(counts);
    return setup_solve(i, power, waist, focal);
}

int ThermalGradBatch::set_temperature(int i, const float *T_host, float power, float waist, float focal) {
    if (i < 0 || i >= count_ || !T_host) {
        set_error("shg_thgrad_set_temperature: bad solve index or null field");
        return SHG_ERR_INVALID;
    }
    TG_TRY(ensure_thermal());
    TG_TRY(ts_->load_temperature(T_host));
    return setup_solve(i, power, waist, focal);
}

int ThermalGradBatch::get_temperature(int i, float *T_host) {
    if (i < 0 || i >= count_ || !ready_[i] || !T_host) {
        set_error("shg_thgrad_get_temperature: solve not set up");
        return SHG_ERR_STATE;
    }
    TG_CUDA(cudaMemcpy(T_host, T_ + (size_t)i * tsize_, tsize_ * sizeof(float), cudaMemcpyDeviceToHost));
    return SHG_OK;
}

static int check_ready(const std::vector<char> &ready);

int ThermalGradBatch::gaussian_pumps(float2 *dst, cudaStream_t st) {
    TG_TRY(check_ready(ready_));
    TG_CUDA(cudaMemcpyAsync(dst, pump0_, (size_t)count_ * nn_ * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    return SHG_OK;
}

// Layout of the work space: in (count*nn), X, cot (count*2nn each), nck checkpoints and
// `slots` states of each of X_s, W_s (count*2nn each; with checkpoints two sets of L, one
// being replayed while the other is reversed; storing every step, L), then 2*count doubles
// of sums.
int ThermalGradBatch::ensure_work(int L, int nck) {
    if (work_ && L == L_ && nck == nck_) return SHG_OK;
    drop_graphs();
    if (work_) cudaFree(work_);
    work_ = nullptr;
    const size_t st = (size_t)count_ * 2 * nn_;
    const size_t slots = (nck > 0 ? 2 : 1) * (size_t)L;
    work_bytes_ = sizeof(float2) * ((size_t)count_ * nn_ + st * (2 + (size_t)nck + 2 * slots)) +
                  sizeof(double) * 2 * (size_t)count_;
    TG_TRY(device_fits(work_bytes_, "batched THERMAL gradient work space"));
    TG_CUDA(cudaMalloc(&work_, work_bytes_));
    float2 *p = static_cast<float2 *>(work_);
    in_ = p;
    p += (size_t)count_ * nn_;
    X_ = p;
    p += st;
    cot_ = p;
    p += st;
    ck_ = p;
    p += st * nck;
    Xs_ = p;
    p += st * slots;
    Ws_ = p;
    p += st * slots;
    sums_ = reinterpret_cast<double *>(p);
    L_ = L;
    nck_ = nck;
    return SHG_OK;
}

// The pass on `st`: input pumps from in_ (SH start zero), K steps forward (saving the
// segment states), losses, and with `grad` the reverse sweep to the pump cotangents in
// the P half of cot_.
int ThermalGradBatch::enqueue(bool grad, int L, int nseg, bool store_all, cudaStream_t st) {
    const int n = n_, K = K_, B = count_, nn = (int)nn_;
    const size_t sz = (size_t)B * 2 * nn_;
    int &nl = launches_;
    nl = 0;
    TG_CUDA(cudaMemsetAsync(sums_, 0, 2 * (size_t)B * sizeof(double), st));
    TG_CUDA(cudaMemcpy2DAsync(X_, 2 * nn_ * sizeof(float2), in_, nn_ * sizeof(float2), nn_ * sizeof(float2), B,
                              cudaMemcpyDeviceToDevice, st));
    TG_CUDA(cudaMemset2DAsync(X_ + nn_, 2 * nn_ * sizeof(float2), 0, nn_ * sizeof(float2), B, st));
    TG_CUDA(launch_abs2_sum_b(X_, nn, 0, sums_ + B, B, st));
    ++nl;
    auto diffraction = [&](float2 *A, int mode, cudaStream_t q) -> int {
        TG_CUDA(launch_dft_rows(n, +1, A, A, q, 2 * B));
        TG_CUDA(launch_colpass(n, mode, A, nullptr, d_desc_, nullptr, q, B));
        TG_CUDA(launch_dft_rows(n, -1, A, A, q, 2 * B));
        nl += 3;
        return SHG_OK;
    };
    // Step boundary s (0 <= s <= K) of the forward march on X_: second RK4 of step s-1
    // (input W_{s-1} to save_w), X_s to save_x, first RK4 of step s; one pass per boundary.
    auto boundary = [&](int s, int s_end, float2 *save_w, float2 *save_x, cudaStream_t q) -> int {
        TG_CUDA(launch_th_rk4_pair(X_, save_w, save_x, coef_, nn, K, s - 1, s < s_end ? s : -1, d_desc_, B, q));
        ++nl;
        return SHG_OK;
    };
    // Checkpointed: segment seg's states go to slot set seg & 1 (replayed there, or, for the
    // last two segments, written by the forward pass itself, which the two slot sets hold
    // without a replay)
    auto slot_set = [&](int seg) -> size_t { return (size_t)(seg & 1) * L * sz; };
    auto stored = [&](int seg) -> bool { return !store_all && seg >= nseg - 2; };
    // forward from the inputs: checkpoints every L steps (store_all: X_s, W_s of every step;
    // checkpointed: X_s, W_s of the last two segments as well)
    auto save_x = [&](int s) -> float2 * {
        if (!grad || s >= K) return nullptr;
        if (store_all) return Xs_ + (size_t)s * sz;
        if (stored(s / L)) return Xs_ + slot_set(s / L) + (size_t)(s % L) * sz;
        return s % L == 0 ? ck_ + (size_t)(s / L) * sz : nullptr;
    };
    auto save_w = [&](int s) -> float2 * {
        if (!grad) return nullptr;
        if (store_all) return Ws_ + (size_t)s * sz;
        return stored(s / L) ? Ws_ + slot_set(s / L) + (size_t)(s % L) * sz : nullptr;
    };
    TG_TRY(boundary(0, K, nullptr, save_x(0), st));
    for (int s = 0; s < K; ++s) {
        TG_TRY(diffraction(X_, 0, st));
        TG_TRY(boundary(s + 1, K, save_w(s), save_x(s + 1), st));
    }
    TG_CUDA(launch_abs2_sum_b(X_, nn, nn, sums_, B, st));
    ++nl;
    if (!grad) return SHG_OK;
    TG_CUDA(launch_seed_b(X_, cot_, nn, seed_, B, st));
    ++nl;
    // reverse sweep of steps [s0, s1) on `q` with the states X_s, W_s of those steps at
    // Xs, Ws (slot s - s0): RK4^T at W_{s1-1}; then per step s the adjoint diffraction and
    // one pass with RK4^T at X_s and at W_{s-1}
    auto backward = [&](int s0, int s1, const float2 *Xs, const float2 *Ws, cudaStream_t q) -> int {
        TG_CUDA(launch_th_vjp_pair(nullptr, Ws + (size_t)(s1 - 1 - s0) * sz, cot_, coef_, nn, K, -1, s1 - 1, d_desc_,
                                   B, q));
        ++nl;
        for (int s = s1 - 1; s >= s0; --s) {
            TG_TRY(diffraction(cot_, 2, q));
            const size_t j = (size_t)(s - s0) * sz;
            const bool more = s - 1 >= s0;
            TG_CUDA(launch_th_vjp_pair(Xs + j, more ? Ws + j - sz : nullptr, cot_, coef_, nn, K, s, more ? s - 1 : -1,
                                       d_desc_, B, q));
            ++nl;
        }
        return SHG_OK;
    };
    if (store_all) return backward(0, K, Xs_, Ws_, st);
    // The other segments are replayed from their checkpoints on the side branch into their
    // slot set (X_ is the replay's working state; the reverse sweep works on cot_), so the
    // replay of segment seg-1 runs while segment seg is reversed on `st`.
    auto replay = [&](int seg, cudaStream_t q) -> int {
        const int s0 = seg * L, s1 = std::min(K, s0 + L);
        float2 *Xs = Xs_ + slot_set(seg), *Ws = Ws_ + slot_set(seg);
        TG_CUDA(cudaMemcpyAsync(X_, ck_ + (size_t)seg * sz, sz * sizeof(float2), cudaMemcpyDeviceToDevice, q));
        TG_CUDA(launch_th_rk4_pair(X_, nullptr, Xs, coef_, nn, K, -1, s0, d_desc_, B, q));
        ++nl;
        for (int s = s0; s < s1; ++s) {
            TG_TRY(diffraction(X_, 0, q));
            const size_t j = (size_t)(s - s0) * sz;
            TG_TRY(boundary(s + 1, s1, Ws + j, s + 1 < s1 ? Xs + j + sz : nullptr, q));
        }
        return SHG_OK;
    };
    // branch b waits for everything enqueued so far on branch a
    auto join = [&](cudaStream_t a, cudaStream_t b) -> int {
        TG_CUDA(cudaEventRecord(ev_, a));
        TG_CUDA(cudaStreamWaitEvent(b, ev_, 0));
        return SHG_OK;
    };
    for (int seg = nseg - 1; seg >= 0; --seg) {
        if (!stored(seg)) TG_TRY(join(side_, st));  // replay(seg) done
        // replay(seg-1) reuses the slot set of segment seg+1, whose reverse sweep st finished
        // (and the seed has read the forward's final X_ before the first replay)
        if (seg >= 1 && !stored(seg - 1)) {
            TG_TRY(join(st, side_));
            TG_TRY(replay(seg - 1, side_));
        }
        const int s0 = seg * L, s1 = std::min(K, s0 + L);
        TG_TRY(backward(s0, s1, Xs_ + slot_set(seg), Ws_ + slot_set(seg), st));
    }
    return SHG_OK;
}

int ThermalGradBatch::finish(double *p_sh, double *p_in, cudaStream_t st) {
    if (!p_sh && !p_in) return SHG_OK;
    std::vector<double> s(2 * (size_t)count_);
    TG_CUDA(cudaMemcpyAsync(s.data(), sums_, s.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    for (int b = 0; b < count_; ++b) {
        const float np = crystal_index(cfg_.crystal, cfg_.lp, tc_[b]),
                    ns = crystal_index(cfg_.crystal, (float)(0.5 * (double)cfg_.lp), tc_[b]);
        if (p_sh) p_sh[b] = field_power(s[b], ns, h_desc_[b].dx, h_desc_[b].dy);
        if (p_in) p_in[b] = field_power(s[count_ + b], np, h_desc_[b].dx, h_desc_[b].dy);
    }
    return SHG_OK;
}

static int capture(cudaStream_t cap, cudaGraphExec_t *out, const std::function<int(cudaStream_t)> &body) {
    cudaGraph_t g = nullptr;
    TG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    const int rc = body(cap);
    const cudaError_t e = cudaStreamEndCapture(cap, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    TG_CUDA(e);
    const cudaError_t e2 = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    TG_CUDA(e2);
    return SHG_OK;
}

static int check_ready(const std::vector<char> &ready) {
    for (char r : ready)
        if (!r) {
            set_error("thgrad: every solve needs its temperature field first (solve_temperature / set_temperature)");
            return SHG_ERR_STATE;
        }
    return SHG_OK;
}

int ThermalGradBatch::forward(const float2 *pump_in, float2 *pump_out, float2 *sh_out, double *p_sh, double *p_in,
                              cudaStream_t st) {
    TG_TRY(check_ready(ready_));
    if (!pump_in) {
        set_error("shg_thgrad_forward: pump_in is required");
        return SHG_ERR_INVALID;
    }
    if (!work_) TG_TRY(ensure_work(0, 0));
    if (!g_fwd_) {
        TG_TRY(capture(cap_, &g_fwd_, [&](cudaStream_t c) { return enqueue(false, 1, 0, false, c); }));
        launches_fwd_ = launches_;
    }
    const size_t fb = nn_ * sizeof(float2);
    TG_CUDA(cudaMemcpyAsync(in_, pump_in, (size_t)count_ * fb, cudaMemcpyDeviceToDevice, st));
    TG_CUDA(cudaGraphLaunch(g_fwd_, st));
    launches_ = launches_fwd_;
    if (pump_out) TG_CUDA(cudaMemcpy2DAsync(pump_out, fb, X_, 2 * fb, fb, count_, cudaMemcpyDeviceToDevice, st));
    if (sh_out) TG_CUDA(cudaMemcpy2DAsync(sh_out, fb, X_ + nn_, 2 * fb, fb, count_, cudaMemcpyDeviceToDevice, st));
    return finish(p_sh, p_in, st);
}

int ThermalGradBatch::gradient(const float2 *pump_in, int checkpoints, float2 *grad, double *p_sh, double *p_in,
                               cudaStream_t st) {
    TG_TRY(check_ready(ready_));
    if (!pump_in || !grad) {
        set_error("shg_thgrad_gradient: pump_in and grad are required");
        return SHG_ERR_INVALID;
    }
    const int K = K_;
    if (checkpoints < 1) checkpoints = 1;
    const bool store_all = checkpoints >= K;
    const int L = store_all ? K : (K + checkpoints - 1) / checkpoints;
    const int nseg = store_all ? 1 : (K + L - 1) / L;
    const int nck = store_all ? 0 : nseg;
    // the forward-only graph stays valid for any work-space layout with the same buffers
    if (L != L_ || nck != nck_) TG_TRY(ensure_work(L, nck));
    if (!g_grad_ || g_grad_L_ != L || g_grad_all_ != store_all) {
        if (g_grad_) cudaGraphExecDestroy(g_grad_);
        g_grad_ = nullptr;
        if (!side_) TG_CUDA(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
        if (!ev_) TG_CUDA(cudaEventCreateWithFlags(&ev_, cudaEventDisableTiming));
        TG_TRY(capture(cap_, &g_grad_, [&](cudaStream_t c) { return enqueue(true, L, nseg, store_all, c); }));
        g_grad_L_ = L;
        g_grad_all_ = store_all;
        launches_grad_ = launches_;
    }
    const size_t fb = nn_ * sizeof(float2);
    TG_CUDA(cudaMemcpyAsync(in_, pump_in, (size_t)count_ * fb, cudaMemcpyDeviceToDevice, st));
    TG_CUDA(cudaGraphLaunch(g_grad_, st));
    launches_ = launches_grad_;
    TG_CUDA(cudaMemcpy2DAsync(grad, fb, cot_, 2 * fb, fb, count_, cudaMemcpyDeviceToDevice, st));
    return finish(p_sh, p_in, st);
}

}  // namespace shg

using namespace shg;

struct shg_thgrad {
    ThermalGradBatch b;
};

extern "C" {

int shg_thgrad_create(const shg_config *cfg, int count, shg_thgrad **out) {
    if (!cfg || !out) {
        set_error("shg_thgrad_create: null argument");
        return SHG_ERR_INVALID;
    }
    *out = nullptr;
    shg_thgrad *h = new (std::nothrow) shg_thgrad;
    if (!h) return SHG_ERR_NOMEM;
    const int rc = h->b.create(*cfg, count);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return SHG_OK;
}

void shg_thgrad_destroy(shg_thgrad *h) { delete h; }

int shg_thgrad_solve_temperature(shg_thgrad *h, int i, float power, float waist, float focal, float temp,
                                 float t_inf, float t1, float t2, int *counts) {
    shg::Phase phase("shg_thgrad_solve_temperature");
    if (!h) return SHG_ERR_INVALID;
    return h->b.solve_temperature(i, power, waist, focal, temp, t_inf, t1, t2, counts);
}

int shg_thgrad_set_temperature(shg_thgrad *h, int i, const float *T, float power, float waist, float focal) {
    if (!h) return SHG_ERR_INVALID;
    return h->b.set_temperature(i, T, power, waist, focal);
}

int shg_thgrad_get_temperature(shg_thgrad *h, int i, float *T) {
    if (!h) return SHG_ERR_INVALID;
    return h->b.get_temperature(i, T);
}

int shg_thgrad_gaussian_pumps(shg_thgrad *h, void *pump, void *stream) {
    if (!h || !pump) return SHG_ERR_INVALID;
    return h->b.gaussian_pumps(static_cast<float2 *>(pump), static_cast<cudaStream_t>(stream));
}

int shg_thgrad_forward(shg_thgrad *h, const void *pump_in, void *pump_out, void *sh_out, double *p_sh, double *p_in,
                       void *stream) {
    shg::Phase phase("shg_thgrad_forward");
    if (!h) return SHG_ERR_INVALID;
    return h->b.forward(static_cast<const float2 *>(pump_in), static_cast<float2 *>(pump_out),
                        static_cast<float2 *>(sh_out), p_sh, p_in, static_cast<cudaStream_t>(stream));
}

int shg_thgrad_gradient(shg_thgrad *h, const void *pump_in, int checkpoints, void *grad_pump, double *p_sh,
                        double *p_in, void *stream) {
    shg::Phase phase("shg_thgrad_gradient");
    if (!h) return SHG_ERR_INVALID;
    return h->b.gradient(static_cast<const float2 *>(pump_in), checkpoints, static_cast<float2 *>(grad_pump), p_sh,
                         p_in, static_cast<cudaStream_t>(stream));
}

int shg_thgrad_launch_count(const shg_thgrad *h) { return h ? h->b.launches() : -1; }

double shg_thgrad_device_bytes(const shg_thgrad *h) { return h ? (double)h->b.device_bytes() : 0.0; }

}  // extern "C"
