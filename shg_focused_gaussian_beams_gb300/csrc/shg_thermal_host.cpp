// THERMAL solve on the device: Solver::run with -DTHERMAL (Solver.h:287-340) and its
// components. Compiled with -ffp-contract=off: the heat-stencil coefficients keep the
// reference's float rounding (Tfield.h:118-125).
#include "shg_thermal_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <map>
#include <mutex>
#include <random>
#include <utility>
#include <string>

#include "../../include/shg.h"

namespace shg {

#define TH_CUDA(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                            \
            return e_ == cudaErrorMemoryAllocation ? SHG_ERR_NOMEM : SHG_ERR_CUDA;                     \
        }                                                                                              \
    } while (0)

#define TH_TRY(expr)         \
    do {                     \
        int rc_ = (expr);    \
        if (rc_) return rc_; \
    } while (0)

HeatCoef make_heat_coef(const shg_config &cfg, float T_inf) {
    HeatCoef c;
    std::memset(&c, 0, sizeof(c));
    const float dx = cfg.lx / (float)(unsigned)(cfg.nx - 1);
    const float dy = cfg.ly / (float)(unsigned)(cfg.ny - 1);
    const float dz = cfg.lz / (float)(unsigned)(cfg.nz - 1);
    const float k = cfg.kth, h = cfg.htc;
    c.Bix = h * dx / k;
    c.Biy = h * dy / k;
    c.Biz = h * dz / k;
    c.ax = dx * dx / (2 * dy * dy);
    c.ay = dy * dy / (2 * dx * dx);
    c.az = dz * dz / (2 * dx * dx);
    c.bx = dx * dx / (2 * dz * dz);
    c.by = dy * dy / (2 * dz * dz);
    c.bz = dz * dz / (2 * dy * dy);
    c.av = dz / (2 * dx);
    c.bv = dx / (2 * dz);
    c.cv = dx * dz / (4 * dy * dy);
    c.V = (float)(1 / ((double)(c.av + c.bv + 2 * c.cv) + 0.5 * (double)(c.Bix + c.Biz)));
    c.ah = dz / (2 * dy);
    c.bh = dy / (2 * dz);
    c.ch = dy * dz / (4 * dx * dx);
    c.H = (float)(1 / ((double)(c.ah + c.bh + 2 * c.ch) + 0.5 * (double)(c.Biy + c.Biz)));
    c.ad = dx / (2 * dy);
    c.bd = dy / (2 * dx);
    c.cd = dx * dy / (4 * dz * dz);
    c.D = (float)(1 / ((double)(c.ad + c.bd + 2 * c.cd) + 0.5 * (double)(c.Bix + c.Biy)));
    c.AV = dy * dz / dx;
    c.BV = dx * dz / dy;
    c.CV = dx * dy / dz;
    c.BiD = c.Bix * dy + c.Biy * dz + c.Biz * dx;
    c.GV = 1 / (c.AV + c.BV + c.CV + c.BiD);
    c.L2 = 1 / (2 / (dx * dx) + 2 / (dy * dy) + 2 / (dz * dz));
    c.dx2 = dx * dx;
    c.dy2 = dy * dy;
    c.dz2 = dz * dz;
    c.den_x = 1 + 2 * c.ax + 2 * c.bx + c.Bix;
    c.den_y = 1 + 2 * c.ay + 2 * c.by + c.Biy;
    c.den_z = 1 + 2 * c.az + 2 * c.bz + c.Biz;
    c.tinf = T_inf;
    c.KV = 0.5 * (double)T_inf * (double)(c.Bix + c.Biz);
    c.KH = 0.5 * (double)T_inf * (double)(c.Biy + c.Biz);
    c.KD = 0.5 * (double)T_inf * (double)(c.Bix + c.Biy);
    c.tinfBix = c.Bix * T_inf;
    c.tinfBiy = c.Biy * T_inf;
    c.tinfBiz = c.Biz * T_inf;
    c.tinfBiD = T_inf * c.BiD;
    return c;
}

int enable_fast_division(HeatCoef &c, cudaStream_t st) {
    static std::mutex mu;
    static std::map<std::pair<int, unsigned>, bool> verified;  // (device, divisor bits) -> exact
    static std::map<int, unsigned long long *> counters;
    c.rdx2 = 1.0f / c.dx2;
    c.rdy2 = 1.0f / c.dy2;
    c.rdz2 = 1.0f / c.dz2;
    c.fast_div = 0;
    if (std::getenv("SHG_HEAT_DIV") && std::string(std::getenv("SHG_HEAT_DIV")) == "ieee") return SHG_OK;
    int dev = 0;
    TH_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    bool all = true;
    for (float d : {c.dx2, c.dy2, c.dz2}) {
        unsigned bits;
        std::memcpy(&bits, &d, sizeof(bits));
        auto key = std::make_pair(dev, bits);
        auto it = verified.find(key);
        if (it == verified.end()) {
            unsigned long long *&cnt = counters[dev];
            if (!cnt) TH_CUDA(cudaMalloc(&cnt, sizeof(unsigned long long)));
            unsigned long long bad = 1;
            TH_CUDA(verify_fast_division(d, 1.0f / d, cnt, &bad, st));
            it = verified.emplace(key, bad == 0).first;
        }
        all = all && it->second;
    }
    c.fast_div = all ? 1 : 0;
    return SHG_OK;
}

ThermalSolve::~ThermalSolve() {
    for (float *p : {T_[0], T_[1], qk_, np_, ns_, dk_, dkint_})
        if (p) cudaFree(p);
    if (f_) cudaFree(f_);
    if (stepc_) cudaFree(stepc_);
    if (acc_) cudaFree(acc_);
    if (d_desc_) cudaFree(d_desc_);
    if (st_) cudaStreamDestroy(st_);
}

int ThermalSolve::create(const shg_config &cfg) {
    cfg_ = cfg;
    n_ = cfg.nx;
    nz_ = cfg.nz;
    bc_ = cfg.bc;
    sh_seed_ = cfg.sh_seed;
    tsize_ = (size_t)n_ * n_ * nz_;
    const size_t nn = (size_t)n_ * n_;
    TH_CUDA(cudaSetDevice(cfg.device));
    TH_TRY(ensure_twiddles(cfg.device));
    TH_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    for (float **p : {&T_[0], &T_[1], &qk_, &np_, &ns_, &dk_}) TH_CUDA(cudaMalloc(p, tsize_ * sizeof(float)));
    TH_CUDA(cudaMalloc(&dkint_, nn * sizeof(float)));
    TH_CUDA(cudaMalloc(&f_, 6 * nn * sizeof(float2)));
    TH_CUDA(cudaMalloc(&stepc_, (size_t)nz_ * sizeof(float4)));
    // [0..3] power sums, [4] list entry, [5..6] residual sums, [7] the error word (an int,
    // or-ed with 1 by a TMA pipeline wait that gave up, with 2 by a grid-barrier wait of the
    // persistent march that gave up; read with the residual sums), [8] the persistent march's
    // arrival counter
    TH_CUDA(cudaMalloc(&acc_, 9 * sizeof(double)));
    TH_CUDA(cudaMalloc(&d_desc_, sizeof(InstDesc)));
    TH_CUDA(cudaMemset(qk_, 0, tsize_ * sizeof(float)));
    TH_CUDA(cudaMemset(acc_, 0, 9 * sizeof(double)));
    scratch_sum_ = acc_ + 5;
    err_ = reinterpret_cast<int *>(acc_ + 7);
    coop_bar_ = reinterpret_cast<unsigned *>(acc_ + 8);
    return SHG_OK;
}

// Reports and clears a set error word (read beside the residual sums in `words`).
int ThermalSolve::check_error_word(const double *words) {
    int flag = 0;
    std::memcpy(&flag, words, sizeof(int));
    if (!flag) return SHG_OK;
    TH_CUDA(cudaMemsetAsync(err_, 0, sizeof(int), st_));
    TH_CUDA(cudaStreamSynchronize(st_));
    set_error((flag & 1) ? "heat sweep: a TMA pipeline wait gave up (sweep incomplete)"
                         : "THERMAL march: a grid-barrier wait of the persistent launch gave up (march incomplete)");
    return SHG_ERR_CUDA;
}

// The THERMAL march as one persistent cooperative launch where its grid fits co-resident
// (SHG_THERMAL_MARCH=streaming keeps the two launches per z-step), decided once.
bool ThermalSolve::use_coop() {
    if (coop_ < 0) {
        const char *m = std::getenv("SHG_THERMAL_MARCH");
        const bool want = !(m && std::string(m) == "streaming");
        coop_ = want && launch_coop_th(n_, nullptr, th_, nullptr, nullptr, nullptr) == cudaSuccess ? 1 : 0;
        cudaGetLastError();
    }
    return coop_ == 1;
}

int ThermalSolve::sq_diff(float *out) {
    double w[3] = {0.0, 0.0, 0.0};  // residual sum, (unused), error word
    TH_CUDA(launch_sq_diff_sum(T_cur(), T_prev(), tsize_, scratch_sum_, st_));
    TH_CUDA(cudaMemcpyAsync(w, scratch_sum_, sizeof(w), cudaMemcpyDeviceToHost, st_));
    TH_CUDA(cudaStreamSynchronize(st_));
    TH_TRY(check_error_word(w + 2));
    *out = (float)w[0] / (float)(unsigned)tsize_;
    return SHG_OK;
}

int ThermalSolve::sweeps(float t_inf, int n) {
    if (t_inf != tinf_coef_) {
        hc_ = make_heat_coef(cfg_, t_inf);
        TH_TRY(enable_fast_division(hc_, st_));
        tinf_coef_ = t_inf;
    }
    const int L = heat_levels();
    for (; L > 1 && n >= L; n -= L) {
        TH_CUDA(launch_heat_tb(T_[cur_ ^ 1], T_[cur_], qk_, hc_, n_, n_, nz_, bc_, L, st_));
        cur_ ^= 1;
    }
    for (int k = 0; k < n; ++k) {
        TH_CUDA(launch_heat(T_[cur_ ^ 1], T_[cur_], qk_, hc_, n_, n_, nz_, bc_, err_, st_));
        cur_ ^= 1;
    }
    return SHG_OK;
}

// A TMA-staged sweep whose pipeline gave up leaves its error word set: report it.
static int heat_pipeline_ok(int *err, cudaStream_t st) {
    int flag = 0;
    TH_CUDA(heat_tma_error(err, &flag, st));
    if (flag) {
        set_error("heat sweep: a TMA pipeline wait gave up (sweep incomplete)");
        return SHG_ERR_CUDA;
    }
    return SHG_OK;
}

int ThermalSolve::sweeps_checked(float t_inf, int n) {
    TH_TRY(sweeps(t_inf, n));
    return heat_pipeline_ok(err_, st_);
}

// Solver.h:302-324: the residual is checked after the first sweep and then after every
// 5000th; the loop stops when it is below 5e-4/TSIZE or equal to the previous check. The
// error word is read at every residual check, so a sweep whose pipeline gave up ends the
// solve there (its stale voxels could otherwise keep the residual above the tolerance).
int ThermalSolve::jacobi(float t_inf, int *counter) {
    shg::Phase phase("Jacobi solve");
    const int rc = jacobi_run(t_inf, counter);
    if (rc) return rc;
    return heat_pipeline_ok(err_, st_);
}

int ThermalSolve::jacobi_run(float t_inf, int *counter) {
    if (rel_tol_ > 0) {
        // relative residual of one sweep, every check_every sweeps
        int c = 0;
        double sums[3];  // |T_k+1 - T_k|^2, |T_k+1|^2, error word
        for (;;) {
            const int n = std::min(check_every_ - 1, max_sweeps_ - 1 - c);
            if (n > 0) TH_TRY(sweeps(t_inf, n));
            TH_TRY(sweeps(t_inf, 1));
            c += n + 1;
            TH_CUDA(launch_sq_sums(T_cur(), T_prev(), tsize_, scratch_sum_, st_));
            TH_CUDA(cudaMemcpyAsync(sums, scratch_sum_, sizeof(sums), cudaMemcpyDeviceToHost, st_));
            TH_CUDA(cudaStreamSynchronize(st_));
            TH_TRY(check_error_word(sums + 2));
            last_rel_ = sums[1] > 0 ? std::sqrt(sums[0] / sums[1]) : 0.0;
            if (last_rel_ < rel_tol_ || c >= max_sweeps_) break;
        }
        *counter = c;
        return SHG_OK;
    }
    const float tol = (float)(5e-4 / (double)(unsigned)tsize_);
    float rs = 1.0f, aux = -1.0f;
    unsigned c = 0;
    for (;;) {
        TH_TRY(sweeps(t_inf, 1));
        if (c > 0) aux = rs;
        TH_TRY(sq_diff(&rs));
        if (rs == aux) rs = (float)(0.5 * (double)tol);
        c++;
        if (!(rs >= tol)) break;
        TH_TRY(sweeps(t_inf, 4999));
        c += 4999;
    }
    *counter = (int)c;
    return SHG_OK;
}

int ThermalSolve::tables() {
    const float PI = (float)3.14159265358979323846;
    const float lp = cfg_.lp, ls = (float)(0.5 * (double)lp);
    // PhaseMatching.h:105 -> 41: delta-k and the indices from T.
    TH_CUDA(launch_sellmeier_tables(T_cur(), np_, ns_, dk_, tsize_, lp, ls, 2 * PI, 1 / (cfg_.lambda_qpm), cfg_.crystal,
                                    st_));
    // Efields.h:77,110: pump and propagators use T at the grid centre of slice 0.
    const size_t ic = (size_t)(n_ / 2) * n_ + (size_t)(n_ / 2);
    TH_CUDA(cudaMemcpyAsync(&tc_, T_cur() + ic, sizeof(float), cudaMemcpyDeviceToHost, st_));
    TH_CUDA(cudaStreamSynchronize(st_));
    const float dQ = (float)((2.0 / (double)PI) * (double)cfg_.deff);
    const float C = (float)(299792458 * 1E6 / 1E12), EPS0 = (float)(8.8541878128E-12 * 1E12 / 1E6);
    th_.nx = n_;
    th_.ny = n_;
    th_.nz = nz_;
    th_.NP = np_;
    th_.NS = ns_;
    th_.DK = dk_;
    th_.DKint = dkint_;
    th_.QK = qk_;
    th_.pidq = dQ * PI;
    th_.hpidq = dQ * (PI * 0.5f);
    th_.lp = lp;
    th_.ls = ls;
    th_.qc = (float)(0.5 * (double)C * (double)EPS0);
    th_.alpha_p = cfg_.alpha_p;
    th_.alpha_s = cfg_.alpha_s;
    th_.beta_s = cfg_.beta_s;
    th_.kth = cfg_.kth;
    th_.tpa_c = (float)(0.25 * (double)cfg_.beta_s * (double)EPS0 * (double)C);
    return SHG_OK;
}

int ThermalSolve::load_temperature(const float *T_host) {
    TH_CUDA(cudaMemcpyAsync(T_cur(), T_host, tsize_ * sizeof(float), cudaMemcpyHostToDevice, st_));
    TH_TRY(tables());
    return SHG_OK;
}

int ThermalSolve::cwes(float power, float waist, float focal) {
    shg::Phase phase("THERMAL CWES");
    const size_t nn = (size_t)n_ * n_;
    TH_TRY(tables());
    SolveParams sp{n_, nz_, cfg_.lx, cfg_.ly, power, waist, focal, tc_, tc_, tc_};
    std::memset(&h_desc_, 0, sizeof(h_desc_));
    fill_scalars(cfg_, sp, h_desc_);
    h_desc_.P = f_;
    h_desc_.S = f_ + nn;
    h_desc_.Pout = f_ + 2 * nn;
    h_desc_.Sout = f_ + 3 * nn;
    h_desc_.Hp = f_ + 4 * nn;
    h_desc_.Hs = f_ + 5 * nn;
    h_desc_.stepc = stepc_;
    h_desc_.acc = acc_;
    h_desc_.nsteps = nz_;
    h_desc_.pump_given = 0;
    TH_CUDA(cudaMemcpyAsync(d_desc_, &h_desc_, sizeof(InstDesc), cudaMemcpyHostToDevice, st_));
    TH_CUDA(cudaMemsetAsync(acc_, 0, 4 * sizeof(double), st_));
    TH_CUDA(cudaMemsetAsync(acc_ + 4, 0, sizeof(double), st_));  // solve index 0 for the column pass
    if (sh_seed_ >= 0) {
        std::vector<float2> nz(nn);
        std::default_random_engine generator((unsigned)sh_seed_);
        std::normal_distribution<float> distribution(0.0, 1.0e-20);
        for (size_t i = 0; i < nn; ++i) {
            const float a1 = distribution(generator);
            const float a2 = distribution(generator);
            nz[i] = make_float2(a1, a2);
        }
        TH_CUDA(cudaMemcpyAsync(h_desc_.S, nz.data(), nn * sizeof(float2), cudaMemcpyHostToDevice, st_));
        TH_CUDA(cudaStreamSynchronize(st_));
    } else {
        TH_CUDA(cudaMemsetAsync(h_desc_.S, 0, nn * sizeof(float2), st_));
    }
    h_desc_.slices = slices_;
    TH_CUDA(cudaMemcpyAsync(d_desc_, &h_desc_, sizeof(InstDesc), cudaMemcpyHostToDevice, st_));
    TH_CUDA(launch_setup(d_desc_, 1, (int)nn, nz_, st_));
    if (slices_) {
        TH_CUDA(cudaMemcpyAsync(slices_, h_desc_.P, nn * sizeof(float2), cudaMemcpyDeviceToDevice, st_));
        TH_CUDA(cudaMemcpyAsync(slices_ + nn, h_desc_.S, nn * sizeof(float2), cudaMemcpyDeviceToDevice, st_));
    }
    if (use_coop()) {
        TH_CUDA(cudaMemsetAsync(coop_bar_, 0, sizeof(unsigned), st_));
        TH_CUDA(launch_coop_th(n_, d_desc_, th_, coop_bar_, err_, st_));
        return SHG_OK;
    }
    const int *list0 = reinterpret_cast<const int *>(acc_ + 4);
    for (int s = 0; s <= nz_; ++s) {
        TH_CUDA(launch_rows_th(n_, d_desc_, th_, s, st_));
        if (s < nz_) TH_CUDA(launch_cols(n_, d_desc_, list0, 1, st_));
    }
    return SHG_OK;
}

int ThermalSolve::run(float power, float waist, float focal, float temp, float t_inf, float t1, float t2) {
    temp_ = temp;
    for (int i = 0; i < 5; ++i) counts_[i] = -1;
    // Solver.h:287-293
    TH_CUDA(launch_init_temperature(T_[0], n_, n_, nz_, temp, t1, t2, bc_, st_));
    TH_CUDA(cudaMemcpyAsync(T_[1], T_[0], tsize_ * sizeof(float), cudaMemcpyDeviceToDevice, st_));
    TH_CUDA(cudaMemsetAsync(qk_, 0, tsize_ * sizeof(float), st_));
    cur_ = 0;
    unsigned global_count = 0, num_of_iter = 5;
    int outer = 0;
    while (global_count < num_of_iter) {
        int counter = 0;
        TH_TRY(jacobi(t_inf, &counter));
        counts_[outer++] = counter;
        TH_TRY(cwes(power, waist, focal));
        if (counter == 1 && global_count != 0) global_count = num_of_iter;
        global_count++;
    }
    // the error word once more: a persistent march that gave up in the last CWES
    double w = 0.0;
    TH_CUDA(cudaMemcpyAsync(&w, acc_ + 7, sizeof(double), cudaMemcpyDeviceToHost, st_));
    TH_CUDA(cudaStreamSynchronize(st_));
    TH_TRY(check_error_word(&w));
    have_result_ = true;
    return SHG_OK;
}

int ThermalSolve::copy_temperature(float *T_host) {
    TH_CUDA(cudaStreamSynchronize(st_));
    TH_CUDA(cudaMemcpy(T_host, T_cur(), tsize_ * sizeof(float), cudaMemcpyDeviceToHost));
    return SHG_OK;
}

int ThermalSolve::copy_fields(float *pump, float *sh) {
    const size_t nn = (size_t)n_ * n_;
    TH_CUDA(cudaStreamSynchronize(st_));
    if (pump) TH_CUDA(cudaMemcpy(pump, f_ + 2 * nn, nn * sizeof(float2), cudaMemcpyDeviceToHost));
    if (sh) TH_CUDA(cudaMemcpy(sh, f_ + 3 * nn, nn * sizeof(float2), cudaMemcpyDeviceToHost));
    return SHG_OK;
}

int ThermalSolve::powers(double *pin, double *psh, double *pout) {
    double acc[4];
    TH_CUDA(cudaStreamSynchronize(st_));
    TH_CUDA(cudaMemcpy(acc, acc_, sizeof(acc), cudaMemcpyDeviceToHost));
    const float np_c = crystal_index(cfg_.crystal, cfg_.lp, tc_),
                ns_c = crystal_index(cfg_.crystal, (float)(0.5 * (double)cfg_.lp), tc_);
    const float dx = cfg_.lx / (float)(unsigned)(n_ - 1), dy = cfg_.ly / (float)(unsigned)(n_ - 1);
    if (pin) *pin = field_power(acc[0], np_c, dx, dy);
    if (psh) *psh = field_power(acc[1], ns_c, dx, dy);
    if (pout) *pout = field_power(acc[2], np_c, dx, dy);
    return SHG_OK;
}

}  // namespace shg

using namespace shg;

namespace {

int thermal_component_cfg(const shg_config *cfg) {
    if (!cfg) {
        set_error("null config");
        return SHG_ERR_INVALID;
    }
    if (cfg->nx < 2 || cfg->ny < 2 || cfg->nz < 2) {
        set_error("grid sizes must be > 1");
        return SHG_ERR_INVALID;
    }
    if (cfg->nx != cfg->ny) {
        set_error("the device thermal path needs NX = NY");
        return SHG_ERR_UNSUPPORTED;
    }
    if (cfg->crystal != SHG_CRYSTAL_SPPLT && cfg->crystal != SHG_CRYSTAL_PPLN) {
        set_error("crystal must be SHG_CRYSTAL_SPPLT or SHG_CRYSTAL_PPLN");
        return SHG_ERR_INVALID;
    }
    return SHG_OK;
}

}  // namespace

extern "C" {

int shg_init_temperature(const shg_config *cfg, float temp, float t1, float t2, int bc, float *T_out) {
    TH_TRY(thermal_component_cfg(cfg));
    ThermalSolve ts;
    shg_config c = *cfg;
    c.bc = bc;
    TH_TRY(ts.create(c));
    TH_CUDA(launch_init_temperature(ts.T_cur(), c.nx, c.ny, c.nz, temp, t1, t2, bc, ts.stream()));
    return ts.copy_temperature(T_out);
}

int shg_heat_sweeps(const shg_config *cfg, float *T_inout, const float *Q, float t_inf, int nsweeps, int bc) {
    TH_TRY(thermal_component_cfg(cfg));
    if (!T_inout || !Q || nsweeps < 0) {
        set_error("shg_heat_sweeps: bad argument");
        return SHG_ERR_INVALID;
    }
    ThermalSolve ts;
    shg_config c = *cfg;
    c.bc = bc;
    TH_TRY(ts.create(c));
    const size_t n = ts.tsize();
    // Tfield.h:132 divides Q by the conductivity per voxel and sweep; the quotient is
    // formed once here with the same float division.
    std::vector<float> qk(n);
    for (size_t i = 0; i < n; ++i) qk[i] = Q[i] / c.kth;
    TH_CUDA(cudaMemcpy(ts.QK(), qk.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    TH_CUDA(cudaMemcpy(ts.T_cur(), T_inout, n * sizeof(float), cudaMemcpyHostToDevice));
    TH_CUDA(cudaMemcpy(ts.T_prev(), T_inout, n * sizeof(float), cudaMemcpyHostToDevice));
    TH_TRY(ts.sweeps_checked(t_inf, nsweeps));
    return ts.copy_temperature(T_inout);
}

int shg_heat_sweeps_device(const shg_config *cfg, void *Ta, void *Tb, const void *QK, float t_inf, int nsweeps, int bc,
                           void *stream) {
    TH_TRY(thermal_component_cfg(cfg));
    if (!Ta || !Tb || !QK || nsweeps < 0) {
        set_error("shg_heat_sweeps_device: bad argument");
        return SHG_ERR_INVALID;
    }
    HeatCoef hc = make_heat_coef(*cfg, t_inf);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    TH_TRY(enable_fast_division(hc, st));
    // this call's own error word, leased from a pool (no other call can set or clear it)
    int *err = nullptr;
    TH_CUDA(heat_error_word_acquire(&err));
    struct Lease {
        int *w;
        ~Lease() { heat_error_word_release(w); }
    } lease{err};
    float *a = static_cast<float *>(Ta), *b = static_cast<float *>(Tb);
    const int L = heat_levels();
    for (; L > 1 && nsweeps >= L; nsweeps -= L) {
        TH_CUDA(launch_heat_tb(b, a, static_cast<const float *>(QK), hc, cfg->nx, cfg->ny, cfg->nz, bc, L, st));
        std::swap(a, b);
    }
    for (int k = 0; k < nsweeps; ++k) {
        TH_CUDA(launch_heat(b, a, static_cast<const float *>(QK), hc, cfg->nx, cfg->ny, cfg->nz, bc, err, st));
        std::swap(a, b);
    }
    // heat_pipeline_ok synchronises `st` and clears the word before it returns to the pool
    return heat_pipeline_ok(err, st);
}

int shg_dk_thermal(const shg_config *cfg, const float *T, float *DK, float *NP, float *NS) {
    TH_TRY(thermal_component_cfg(cfg));
    ThermalSolve ts;
    TH_TRY(ts.create(*cfg));
    const size_t n = ts.tsize();
    std::vector<float> tmp(3 * n);
    float *d = nullptr;
    TH_CUDA(cudaMalloc(&d, 3 * n * sizeof(float)));
    const float PI = (float)3.14159265358979323846;
    const float lp = cfg->lp, ls = (float)(0.5 * (double)lp);
    cudaError_t e = cudaMemcpy(ts.T_cur(), T, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_sellmeier_tables(ts.T_cur(), d, d + n, d + 2 * n, n, lp, ls, 2 * PI,
                                                      1 / (cfg->lambda_qpm), cfg->crystal, ts.stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(ts.stream());
    if (e == cudaSuccess) e = cudaMemcpy(tmp.data(), d, 3 * n * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    TH_CUDA(e);
    if (NP) std::memcpy(NP, tmp.data(), n * sizeof(float));
    if (NS) std::memcpy(NS, tmp.data() + n, n * sizeof(float));
    if (DK) std::memcpy(DK, tmp.data() + 2 * n, n * sizeof(float));
    return SHG_OK;
}

}  // extern "C"
