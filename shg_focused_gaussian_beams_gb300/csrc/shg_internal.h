// Internal declarations shared by the CUDA translation units and the host library.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <string>

#include "../../include/shg.h"

namespace shg {

// A named NVTX range over one host-side phase of an entry point (shown by Nsight tools and
// usable as an ncu --nvtx filter); without an attached tool a push or pop is one test of a
// function pointer.
struct Phase {
    explicit Phase(const char *name) { nvtxRangePushA(name); }
    ~Phase() { nvtxRangePop(); }
    Phase(const Phase &) = delete;
    Phase &operator=(const Phase &) = delete;
};

struct InstDesc;

// Device addresses of every translation unit's twiddle-table copy (current device).
const float2 *twiddle_symbol_address_march();
const float2 *twiddle_symbol_address_thermal();
const float2 *twiddle_symbol_address_adjoint();
const float2 *twiddle_symbol_address_resident();
const float2 *twiddle_symbol_address_resident128();
const float2 *twiddle_symbol_address_resident256();
const float2 *twiddle_symbol_address_cluster_pt();

// Check build (shg_check.cuh): each kernel translation unit's first failed check, read and
// cleared (0: none; ~0: unreadable); always 0 in other builds.
unsigned long long check_word_take_march();
unsigned long long check_word_take_resident64();
unsigned long long check_word_take_resident128();
unsigned long long check_word_take_resident256();
unsigned long long check_word_take_cluster_pt();
unsigned long long check_word_take_thermal();
unsigned long long check_word_take_heat_tma();
unsigned long long check_word_take_adjoint();
cudaError_t launch_check_selftest(long long value);

// shg_resident_variants.cu (resident march): variants (cluster size, CTAs per SM) per grid size
struct ResidentVariant {
    int cs, minb, g;  // cluster size, CTAs per SM, threads per line (FFT split N = (N/g) x g);
                      // cs == 0: the persistent cooperative grid of one solve (launch_coop);
                      // cs == -1: one cluster per solve, one thread per point in the
                      // pointwise phase (launch_cluster_pt)
};
int resident_variants(int n, ResidentVariant *out, int max_out);
ResidentVariant resident_default(int n);
cudaError_t prepare_resident(int n, ResidentVariant v, int *max_clusters);
cudaError_t launch_resident(int n, ResidentVariant v, const InstDesc *inst, const int *list, int njobs, int *counter,
                            int max_clusters, cudaStream_t st);

// shg_march.cu
cudaError_t launch_setup(const InstDesc *inst, int n_inst, int max_nn, int max_nz, cudaStream_t st);
cudaError_t launch_rows(int n, const InstDesc *inst, const int *list, int count, int s, cudaStream_t st);
cudaError_t launch_cols(int n, const InstDesc *inst, const int *list, int count, cudaStream_t st);
// The whole march of one solve (list[0]) as one cooperative launch with bounded grid
// barriers (bar: two zeroed words; err: zeroed, set to 1 when a barrier wait gave up).
// inst == nullptr only checks that the grid fits co-resident; blocks receives its size.
cudaError_t launch_coop(int n, const InstDesc *inst, const int *list, unsigned *bar, int *err, cudaStream_t st,
                        int *blocks = nullptr);
bool line_length_supported(int n);

// shg_cluster_pt.cu: the march of each of `count` solves (list[0..count)) in one
// thread-block cluster of cluster_pt_size(n) CTAs, both fields in the cluster's shared
// memory (n in {64, 128, 256}). prepare_cluster_pt: once per device, outside any capture;
// max_clusters receives how many clusters fit at once (0: none).
int cluster_pt_size(int n);
cudaError_t prepare_cluster_pt(int n, int *max_clusters);
cudaError_t launch_cluster_pt(int n, const InstDesc *inst, const int *list, int count, cudaStream_t st);
cudaError_t launch_dft2d(int n, int sign, const float2 *in, float2 *out, cudaStream_t st);
cudaError_t launch_dft_rows(int n, int sign, const float2 *in, float2 *out, cudaStream_t st, int fields = 1);

// shg_thermal.cu
struct HeatCoef;
struct ThermDesc;
cudaError_t launch_init_temperature(float *T, int nx, int ny, int nz, float temp, float t1, float t2, int bc,
                                    cudaStream_t st);
// err: the caller's device error word, set to 1 by the TMA-staged sweep when one of its
// bounded pipeline waits gives up (read and cleared with heat_tma_error).
cudaError_t launch_heat(float *Tf, const float *Ti, const float *QK, const HeatCoef &c, int nx, int ny, int nz,
                        int bc, int *err, cudaStream_t st);
// K = levels sweeps in one launch (temporal blocking), levels in {2, 3, 4}; bit-identical
// to K launch_heat calls. heat_levels(): the level count in use (SHG_HEAT_TB, default 1 =
// no temporal blocking: the sweep is issue-bound, and the blocked form's redundant halo
// updates cost more issue slots than its saved DRAM traffic on GB300).
cudaError_t launch_heat_tb(float *Tf, const float *Ti, const float *QK, const HeatCoef &c, int nx, int ny, int nz,
                           int bc, int levels, cudaStream_t st);
int heat_levels();
cudaError_t verify_fast_division(float d, float r, unsigned long long *d_count, unsigned long long *mismatches,
                                 cudaStream_t st);
// shg_heat_tma.cu: the TMA-staged sweep (NX % 4 == 0) and its pipeline error word. Each
// THERMAL solve owns one device int; component calls lease one from a pool.
bool heat_tma_supported(int nx, int ny, int nz);
cudaError_t launch_heat_tma(float *Tf, const float *Ti, const float *QK, const HeatCoef &c, int nx, int ny, int nz,
                            int bc, int *err, cudaStream_t st, int rows_per_warp = 1);
cudaError_t heat_tma_error(int *err, int *flag, cudaStream_t st);
cudaError_t heat_error_word_acquire(int **err);
void heat_error_word_release(int *err);
cudaError_t launch_sq_diff_sum(const float *Tf, const float *Ti, size_t n, double *out, cudaStream_t st);
cudaError_t launch_sq_sums(const float *Tf, const float *Ti, size_t n, double *out2, cudaStream_t st);
// crystal: SHG_CRYSTAL_SPPLT (Crystal.h:55-71) or SHG_CRYSTAL_PPLN (sellmeier_ln).
cudaError_t launch_sellmeier_tables(const float *T, float *NP, float *NS, float *DK, size_t n, float lp, float ls,
                                    float two_pi, float inv_lambda, int crystal, cudaStream_t st);
cudaError_t launch_rows_th(int n, const InstDesc *d, const ThermDesc &th, int s, cudaStream_t st);
// The whole THERMAL march of one solve (stages 0..nz) as one cooperative launch with bounded
// grid barriers (bar: a zeroed word; err: the solve's error word, or-ed with 2 when a barrier
// wait gave up). d == nullptr only checks that the grid fits co-resident.
cudaError_t launch_coop_th(int n, const InstDesc *d, const ThermDesc &th, unsigned *bar, int *err, cudaStream_t st);

// One solve's run parameters (Solver::run arguments and the temperatures its set-up
// calls read).
struct SolveParams {
    int n, nz;
    float lx, ly;
    float power, waist, focal;
    float temp;   // coupling and phase-mismatch temperature (dAdz, initDKConstant)
    float tpump;  // index temperature of the Gaussian pump (setPump reads T at the grid centre)
    float tprop;  // index temperature of the propagators (beamPropagator, same centre value)
};

// shg_files.cpp (Files.h formats)
bool save_matrix_complex(const std::string &dir, const std::string &name, const float2 *v, int nx, int ny);
bool save_tensor_real(const std::string &dir, const std::string &name, const float *T, int nx, int ny, int nz);

// shg_host.cpp
void set_error(const std::string &msg);
float sellmeier(float L, float T);     // Crystal.h:55-71 (MgO:sPPLT)
float sellmeier_ln(float L, float T);  // PPLN (congruent LiNbO3, Jundt 1997)
float crystal_index(int crystal, float L, float T);
void fill_scalars(const shg_config &cr, const SolveParams &sp, InstDesc &d);
double field_power(double sum_abs2, float n_index, float dx, float dy);
int ensure_twiddles(int device);
int device_fits(size_t bytes, const char *what);

}  // namespace shg
