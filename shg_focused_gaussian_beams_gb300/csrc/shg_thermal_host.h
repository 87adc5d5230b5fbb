// Host orchestration of one THERMAL solve (Solver::run with -DTHERMAL, Solver.h:287-340).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "shg_internal.h"
#include "shg_thermal.cuh"

namespace shg {

// Tfield.h:118-125 coefficients with the reference's rounding.
HeatCoef make_heat_coef(const shg_config &cfg, float t_inf);
// Enables the corrected-product division of the interior stencil when it matches IEEE
// division for every numerator in the checked exponent range, for all three divisors
// (checked once per divisor value on the current device, results cached).
int enable_fast_division(HeatCoef &c, cudaStream_t st);

class ThermalSolve {
   public:
    ~ThermalSolve();
    int create(const shg_config &cfg);
    // Solver::run (THERMAL): temperature set-up, then up to five outer iterations of
    // {Jacobi to the reference's stop rule, delta-k(T), pump and propagators at the centre
    // temperature, CWES with heat-source updates}.
    int run(float power, float waist, float focal, float temp, float t_inf, float t1, float t2);
    int copy_temperature(float *T_host);
    int copy_fields(float *pump, float *sh);
    void counts(int *c) const {
        for (int i = 0; i < 5; ++i) c[i] = counts_[i];
    }
    int powers(double *pin, double *psh, double *pout);
    // Per-slice capture of every CWES (slot 0 = input state); nullptr: off.
    void set_slices(float2 *s) { slices_ = s; }
    bool has_result() const { return have_result_; }

    // Components (device buffers owned here).
    int jacobi(float t_inf, int *counter);   // one Jacobi solve with the configured stop rule
    // Stop rule: rel_tol <= 0 (default) the reference's (Solver.h:302-324); otherwise stop
    // once ||T_k+1 - T_k|| / ||T_k+1|| < rel_tol, checked every check_every sweeps, at most
    // max_sweeps sweeps per solve.
    void set_stop_rule(double rel_tol, int check_every, int max_sweeps) {
        rel_tol_ = rel_tol;
        check_every_ = check_every < 1 ? 1 : check_every;
        max_sweeps_ = max_sweeps < 1 ? 1 : max_sweeps;
    }
    double last_residual() const { return last_rel_; }
    int sweeps(float t_inf, int n);          // n plain sweeps
    int sweeps_checked(float t_inf, int n);  // n sweeps, then the pipeline error word checked
    int cwes(float power, float waist, float focal);  // one thermal CWES from the current T

    // Indices and delta-k of the current T (PhaseMatching.h:41-54), the centre temperature
    // and the coupling constants; run by cwes() first.
    int tables();
    // Replaces the current temperature field (host, NX*NY*NZ) and builds its tables.
    int load_temperature(const float *T_host);
    const float *NP() const { return np_; }
    const float *NS() const { return ns_; }
    const float *DK() const { return dk_; }
    const ThermDesc &therm() const { return th_; }
    float center_temperature() const { return tc_; }

    float *T_cur() { return T_[cur_]; }
    float *T_prev() { return T_[cur_ ^ 1]; }
    float *QK() { return qk_; }
    size_t tsize() const { return tsize_; }
    cudaStream_t stream() const { return st_; }

   private:
    int sq_diff(float *out);
    int check_error_word(const double *words);
    bool use_coop();
    int jacobi_run(float t_inf, int *counter);
    shg_config cfg_{};
    int n_ = 0, nz_ = 0, bc_ = 0;
    size_t tsize_ = 0;
    float *T_[2] = {nullptr, nullptr};
    int cur_ = 0;
    float *qk_ = nullptr, *np_ = nullptr, *ns_ = nullptr, *dk_ = nullptr, *dkint_ = nullptr;
    float2 *f_ = nullptr;   // P, S, Pout, Sout, Hp, Hs
    float4 *stepc_ = nullptr;
    double *acc_ = nullptr, *scratch_sum_ = nullptr;
    int *err_ = nullptr;  // error word of this solve (in acc_): 1 heat sweep, 2 persistent march
    unsigned *coop_bar_ = nullptr;  // arrival counter of the persistent march (in acc_)
    int coop_ = -1;                 // the THERMAL march as one persistent launch: -1 undecided
    InstDesc *d_desc_ = nullptr;
    InstDesc h_desc_{};
    ThermDesc th_{};
    HeatCoef hc_{};
    float tinf_coef_ = -1e30f;
    cudaStream_t st_ = nullptr;
    int counts_[5] = {-1, -1, -1, -1, -1};
    float tc_ = 0.f, temp_ = 0.f;
    bool have_result_ = false;
    int sh_seed_ = -1;
    float2 *slices_ = nullptr;
    double rel_tol_ = 0.0, last_rel_ = -1.0;
    int check_every_ = 100, max_sweeps_ = 1000000;
};

}  // namespace shg
