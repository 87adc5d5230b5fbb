/* ORACLE — test infrastructure only. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load the library built from this header
 * (oracle/_build/liboracle.so); the product never links it.
 *
 * CPU restatement of the reference's SSFM z-march and thermal solve
 * (alfredos84/SHG_Focused_Gaussian_Beams, src/headers/*.h), with the grid and crystal as
 * run-time values instead of compile-time constants. Two precisions:
 *   f32 — the reference's own arithmetic: float storage, the same operation order, and
 *         the same double-precision sub-expressions the reference's mixed literals create
 *         (Sellmeier, two-photon-absorption factor, heat-source terms, edge formulas of
 *         the heat stencil). Compiled with -ffp-contract=off so that x86 and Arm agree.
 *   f64 — the same method in double; the phase mismatch may be forced to a given float
 *         value (the reference's FP32 delta-k), as the FP64 parity runs require.
 * Complex arrays are interleaved re/im in the reference layout IDX(x,y,z) = z*NX*NY +
 * y*NX + x (Common.h:27-29). Temperatures in C, lengths in um.
 */
#ifndef SHG_ORACLE_H
#define SHG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_cfg {
    int nx, ny, nz;
    float lx, ly, lz;   /* crystal window / length, Crystal.h:31-33 */
    float lp;           /* pump wavelength, Crystal.h:26 */
    float deff;         /* Crystal.h:41 */
    float lambda_qpm;   /* Crystal.h:43 */
    float alpha_p, alpha_s, beta_s;  /* Crystal.h:44-46 */
    float rho_p, rho_s; /* Crystal.h:47-48 */
    float kth, htc;     /* Crystal.h:52-53 */
    int crystal;        /* 0: Crystal.h:55-71 (MgO:sPPLT); 1: PPLN, congruent LiNbO3 (Jundt 1997,
                           not in the reference's code) */
} oracle_cfg;

/* Crystal.h:116-132 */
float oracle_n_f32(float L, float T);
double oracle_n_f64(double L, double T);
/* n(L, T) of crystal 0 (the above) or 1 (PPLN: congruent LiNbO3, Jundt, Opt. Lett. 22, 1553 (1997)). */
float oracle_index_f32(int crystal, float L, float T);
double oracle_index_f64(int crystal, double L, double T);

/* Efields.h:74-104 (pump), Efields.h:107-126 + 32-71 (shifted propagators), FP32. */
void oracle_set_pump_f32(const oracle_cfg *c, float power, float focal, float waist, float tc, float *pump);
void oracle_propagators_f32(const oracle_cfg *c, float tc, float *hp, float *hs);
void oracle_set_pump_f64(const oracle_cfg *c, double power, double focal, double waist, double tc, double *pump);
void oracle_propagators_f64(const oracle_cfg *c, double tc, double *hp, double *hs);
/* PhaseMatching.h:57-70 */
float oracle_dk_constant_f32(const oracle_cfg *c, float temp);
double oracle_dk_constant_f64(const oracle_cfg *c, double temp);

/* Solver.h:156-190: one diffraction step of both fields in place. */
void oracle_diffraction_f32(const oracle_cfg *c, float tc, float *pump, float *sh);
/* Unnormalised 2D DFT, FFTW convention (n0 = nx slow, n1 = ny fast). */
void oracle_dft2d_f32(int n0, int n1, int sign, const float *in, float *out);
void oracle_dft2d_f64(int n0, int n1, int sign, const double *in, double *out);

/* Plain CWES (Solver.h:245-276 without THERMAL) from given fields. out_* receive the
 * state at the top of slice nz-1 (the reference's Pump_out/Signal_out), end_* the state
 * after nz steps (either may be NULL). dk: NaN -> computed from temp. */
void oracle_cwes_plain_f32(const oracle_cfg *c, const float *pump, const float *sh, float temp,
                           float dk, float *out_pump, float *out_sh, float *end_pump, float *end_sh);
void oracle_cwes_plain_f64(const oracle_cfg *c, const double *pump, const double *sh, double temp,
                           double dk, double *out_pump, double *out_sh, double *end_pump, double *end_sh);

/* Solver::run without THERMAL (Solver.h:342-348): pump from (power, focal, waist, temp);
 * SH start zero when sh_seed < 0, else seeded N(0, 1e-20) noise (Efields.h:129-144). */
void oracle_run_plain_f32(const oracle_cfg *c, float power, float waist, float focal, float temp,
                          int sh_seed, float *out_pump, float *out_sh);

/* THERMAL pieces (Tfield.h, PhaseMatching.h). bc 0 = open top (Tfield.h:113),
 * bc 1 = oven surrounded (Tfield.h:224). */
void oracle_init_temperature(const oracle_cfg *c, float temp, float t1, float t2, int bc, float *T);
void oracle_heat_sweeps(const oracle_cfg *c, float *T, const float *Q, float t_inf, int nsweeps, int bc);
/* Host threads of the heat sweeps (default 1); the results do not depend on it. */
void oracle_set_threads(int threads);
float oracle_reduced_sum(const oracle_cfg *c, const float *Tf, const float *Ti);
void oracle_dk_thermal(const oracle_cfg *c, const float *T, float *DK);
void oracle_set_q(const oracle_cfg *c, const float *T, const float *pump, const float *sh, int s, float *Q);
/* THERMAL CWES (Solver.h:245-276) from given fields with the temperature field T
 * (NX*NY*NZ) held fixed: n from T per pixel, delta-k from DK3 (NULL: PhaseMatching.h:41-54
 * evaluated in the function's precision), propagators at tc. out_*: state at the top of
 * slice NZ-1. */
void oracle_cwes_thermal_f32(const oracle_cfg *c, const float *T, const float *DK3, const float *pump,
                             const float *sh, float tc, float *out_pump, float *out_sh);
void oracle_cwes_thermal_f64(const oracle_cfg *c, const double *T, const double *DK3, const double *pump,
                             const double *sh, double tc, double *out_pump, double *out_sh);
/* Solver::run with THERMAL (Solver.h:287-340) as the reference drives it; counts[5]
 * receives the Jacobi sweeps of each outer iteration (-1 if not run). Returns the
 * number of outer iterations. */
int oracle_thermal_run(const oracle_cfg *c, float power, float waist, float focal, float temp,
                       float t_inf, float t1, float t2, int bc, int sh_seed, float *out_pump,
                       float *out_sh, float *T_out, int *counts);

/* A sweep of independent plain solves on `threads` host threads (the SHG.sh
 * one-process-per-point loop). eta[i] = P_SH(out) / P_pump(in). Fields are not kept. */
typedef struct oracle_instance {
    int nx, ny, nz;
    float lx, ly;
    float power, waist, temp, focal;
} oracle_instance;
void oracle_sweep_plain(const oracle_cfg *crystal, const oracle_instance *inst, int n, int threads,
                        double *eta);

/* Power of a field, P = 1/2 eps0 c n sum|A|^2 dx dy, in double. */
double oracle_power_f32(const oracle_cfg *c, const float *field, float n_index);

#ifdef __cplusplus
}
#endif

#endif
