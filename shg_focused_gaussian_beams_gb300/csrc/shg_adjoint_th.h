// Batched gradient of the THERMAL z-march with fixed temperature fields: launchers and the
// host driver behind the shg_thgrad_* entry points.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "shg_internal.h"
#include "shg_march.cuh"
#include "shg_thermal.cuh"

namespace shg {

class ThermalSolve;

cudaError_t launch_th_coef_table(const float *NP, const float *NS, const float *DK, float4 *coef, int nn, int K,
                                 const ThermDesc &th, cudaStream_t st);
// Fused step boundaries: forward RK4 of step sp (second call; input saved to save_w), state
// saved to save_x, RK4 of step sn (first call); reverse RK4^T of step sa at Xa then of step
// sb at Wb. A negative step index skips that half.
cudaError_t launch_th_rk4_pair(float2 *X, float2 *save_w, float2 *save_x, const float4 *coef, int nn, int K, int sp,
                               int sn, const InstDesc *d, int solves, cudaStream_t st);
cudaError_t launch_th_vjp_pair(const float2 *Xa, const float2 *Wb, float2 *cot, const float4 *coef, int nn, int K,
                               int sa, int sb, const InstDesc *d, int solves, cudaStream_t st);
cudaError_t launch_abs2_sum_b(const float2 *X, int nn, int off, double *out, int solves, cudaStream_t st);
cudaError_t launch_seed_b(const float2 *X, float2 *cot, int nn, const double *seed, int solves, cudaStream_t st);

// `count` solves on one NX = NY grid, each with its own fixed temperature field. Solve i's
// loss is its SH output power (state at the top of slice NZ-1, as the THERMAL CWES
// captures it); the gradient is taken with respect to its input pump.
class ThermalGradBatch {
   public:
    ~ThermalGradBatch();
    int create(const shg_config &cfg, int count);
    // Solver::run (THERMAL) for solve i with a Gaussian pump; its final temperature field
    // is kept, together with that pump as the solve's reference input.
    int solve_temperature(int i, float power, float waist, float focal, float temp, float t_inf, float t1, float t2,
                          int *counts);
    // Solve i's temperature field given directly (host, NX*NY*NZ) with the Gaussian
    // reference input of (power, waist, focal).
    int set_temperature(int i, const float *T_host, float power, float waist, float focal);
    int get_temperature(int i, float *T_host);
    int gaussian_pumps(float2 *dst, cudaStream_t st);
    int forward(const float2 *pump_in, float2 *pump_out, float2 *sh_out, double *p_sh, double *p_in, cudaStream_t st);
    int gradient(const float2 *pump_in, int checkpoints, float2 *grad, double *p_sh, double *p_in, cudaStream_t st);
    int launches() const { return launches_; }
    size_t device_bytes() const { return fixed_bytes_ + work_bytes_; }

   private:
    int setup_solve(int i, float power, float waist, float focal);
    int ensure_work(int L, int nck);
    int ensure_thermal();
    int enqueue(bool grad, int L, int nseg, bool store_all, cudaStream_t st);
    int finish(double *p_sh, double *p_in, cudaStream_t st);
    void drop_graphs();

    shg_config cfg_{};
    int n_ = 0, nz_ = 0, K_ = 0, count_ = 0;
    size_t nn_ = 0, tsize_ = 0;
    std::unique_ptr<ThermalSolve> ts_;
    // fixed per solve
    float *T_ = nullptr;          // count * tsize
    float4 *coef_ = nullptr;      // count * K * nn: (kp, ks, tpa1, DKint)
    float2 *props_ = nullptr;     // count * 2 * nn: Hp, Hs (shifted, / nn)
    float2 *pump0_ = nullptr;     // count * nn: Gaussian reference inputs
    float4 *stepc_ = nullptr;     // count * nz: set-up scratch
    double *setup_acc_ = nullptr; // count * 4
    double *seed_ = nullptr;      // count: 2 * P_SH per unit sum |S|^2
    InstDesc *d_desc_ = nullptr;  // count
    std::vector<InstDesc> h_desc_;
    std::vector<float> tc_;
    std::vector<char> ready_;
    size_t fixed_bytes_ = 0;
    // work space of one pass
    void *work_ = nullptr;
    size_t work_bytes_ = 0;
    int L_ = -1, nck_ = -1;
    float2 *in_ = nullptr, *X_ = nullptr, *cot_ = nullptr, *ck_ = nullptr, *Xs_ = nullptr, *Ws_ = nullptr;
    double *sums_ = nullptr;      // [0, count) sum |S_out|^2, [count, 2 count) sum |P_in|^2
    cudaStream_t cap_ = nullptr;
    cudaStream_t side_ = nullptr;  // replay branch of the checkpointed gradient graph
    cudaEvent_t ev_ = nullptr;     // joins between the branches (capture time)
    cudaGraphExec_t g_fwd_ = nullptr, g_grad_ = nullptr;
    int g_grad_L_ = -1;
    bool g_grad_all_ = false;
    int launches_ = 0, launches_fwd_ = 0, launches_grad_ = 0;
};

}  // namespace shg
