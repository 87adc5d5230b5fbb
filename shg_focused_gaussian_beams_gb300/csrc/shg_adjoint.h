// Adjoint z-march: device launchers and the host driver.
#pragma once

#include <cuda_runtime.h>

#include "shg_internal.h"
#include "shg_march.cuh"

namespace shg {

// Column pass of the diffraction over `solves` solves (d[solves], fields solve-major):
// mode 0 forward (spectra into F when F != nullptr), 1 adjoint with the propagator
// sums into acc[2*solves], 2 adjoint without sums.
cudaError_t launch_colpass(int n, int mode, float2 *A, float2 *F, const InstDesc *d, double *acc, cudaStream_t st,
                           int solves = 1);
// Fused row passes of one solve (one row launch per step boundary, see shg_adjoint.cu):
// forward at boundary s (finish the diffraction of step s-1 and RK4 into X_s, or take X_s
// from inP / inS; store W_{s-1}, X_s where asked; RK4 and start step s, or store X_K);
// backward at boundary s (finish the adjoint diffraction of step s+1 and RK4^T at X_{s+1},
// or take the cotangent from C; RK4^T at W_s and start the adjoint diffraction of step s, or
// store the cotangent). States and cotangents hold the pump then the SH field.
cudaError_t launch_adj_rows_fwd(int n, const InstDesc *d, float2 *A, int s, int finish, int start, const float2 *inP,
                                const float2 *inS, float2 *w_out, float2 *x_out, float2 *ck_out, float2 *final_out,
                                cudaStream_t st);
cudaError_t launch_adj_rows_bwd(int n, const InstDesc *d, float2 *C, int s, int finish, int start, const float2 *Xn,
                                const float2 *Wn, double *acc_fin, double *acc_start, cudaStream_t st);
cudaError_t launch_abs2_sum(const float2 *S, int nn, double *out, cudaStream_t st);
cudaError_t launch_seed_cotangent(const float2 *S, float2 *cP, float2 *cS, int nn, const double *g, cudaStream_t st);
// out[0..4) = sum Re(conj(g) dA/dtheta) for theta = focal point, waist, power, pump index,
// where A = (Gaussian pump of Efields.h:74-104) * factor (factor NULL: 1); FP64.
cudaError_t launch_pump_param_sums(const float2 *g, const float2 *factor, int n, float uX, float uY, float dx, float dy,
                                   double ap0, double zr, double w, double f, double power, double nidx, double *out,
                                   cudaStream_t st);
cudaError_t launch_cmul_inplace(float2 *A, const float2 *factor, int nn, cudaStream_t st);

// Device work space of one gradient pass.
struct AdjointWork {
    ~AdjointWork();
    int ensure(int n, int K, int L, int nck);
    void release();
    int n = 0, K = 0, L = 0, nck = 0;
    cudaGraphExec_t graph = nullptr;  // the captured gradient pass for (n, K, L) and graph_key
    cudaStream_t cap = nullptr;       // capture stream
    cudaStream_t side = nullptr;      // second branch of the captured pass (segment replays)
    cudaEvent_t ev = nullptr;         // fork / join of the two branches
    const void *graph_key[4] = {};    // device descriptor, P, S, step constants it was captured on
    void *mem = nullptr;
    size_t bytes = 0;
    float2 *X = nullptr, *cot = nullptr, *ck = nullptr, *Xs = nullptr, *Ws = nullptr, *Fs = nullptr;
    double *acc_step = nullptr, *acc_glob = nullptr;
};

// One gradient pass of the solve described by (h host copy, d device copy) whose P / S
// hold the input fields and whose propagators / step constants are set up. out[0] = loss
// (SH output power, W), out[1] = dL/dT, out[2] = dL/dLambda, out[3] = dL/d(delta k).
int adjoint_run(const shg_config &cfg, const InstDesc &h, const InstDesc *d, float temp, int checkpoints,
                AdjointWork &w, cudaStream_t st, float2 *grad_pump, float2 *grad_sh, double *out);
// After adjoint_run for an input pump A = (Gaussian of (power, waist, focal) at index
// temperature temp) * factor: out4 = dL/dfocal, dL/dwaist, dL/dpower, dL/dT through the
// pump's index n_p(T) (setPump evaluates n at the run temperature).
int pump_param_gradients(const shg_config &cfg, const InstDesc &h, float power, float waist, float focal, float temp,
                         const float2 *factor, AdjointWork &w, cudaStream_t st, double *out4);
double sellmeier_dT(double L, double T);
double crystal_index_dT(int crystal, double L, double T);

}  // namespace shg
