/* shg_gb300 — C ABI of the GB300 SSFM z-march for focused-Gaussian-beam SHG.
 *
 * Drop-in boundary for the reference's solver path (alfredos84/SHG_Focused_Gaussian_Beams,
 * src/headers/Solver.h and the setup classes it drives). Every entry point returns an
 * int status (SHG_OK = 0); shg_last_error() gives the message of the last failure on the
 * calling thread. Plain pointers and sizes only. Complex fields are interleaved float
 * re/im in the reference layout IDX(x, y) = y*NX + x (Common.h:27-29); temperature
 * tensors are float IDX(x, y, z) = z*NX*NY + y*NX + x. Lengths in um, temperatures in C,
 * powers in W (Crystal.h:19-21).
 */
#ifndef SHG_GB300_H
#define SHG_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SHG_OK 0
#define SHG_ERR_INVALID 1      /* bad argument or configuration */
#define SHG_ERR_UNSUPPORTED 2  /* valid for the reference, not implemented on the device */
#define SHG_ERR_CUDA 3         /* CUDA runtime error */
#define SHG_ERR_NOMEM 4        /* device or host allocation failed */
#define SHG_ERR_STATE 5        /* call order (e.g. fields requested before a run) */
#define SHG_ERR_NONFINITE 6    /* a result is NaN or infinite */

/* Grid, crystal and run options. Replaces the compile-time constants of SHG.cpp:11-20
 * and Crystal.h:26-53 and the -DTHERMAL switch (SHG.sh:20-23). */
typedef struct shg_config {
    int nx, ny, nz;          /* SHG.cpp:11-13 */
    float lx, ly, lz;        /* Crystal.h:31-33: window width, height, crystal length */
    float lp;                /* Crystal.h:26: pump wavelength (SH at lp/2) */
    float deff;              /* Crystal.h:41 (dQ = 2/pi * deff, Crystal.h:42) */
    float lambda_qpm;        /* Crystal.h:43: poling period */
    float alpha_p, alpha_s;  /* Crystal.h:44-45: linear absorption, 1/um */
    float beta_s;            /* Crystal.h:46: SH two-photon absorption, um/W */
    float rho_p, rho_s;      /* Crystal.h:47-48: walk-off angles, rad */
    float kth, htc;          /* Crystal.h:52-53: thermal conductivity, heat-transfer coefficient */
    int thermal;             /* 1 = the -DTHERMAL build (Solver.h:289-340) */
    int bc;                  /* 0 = open top, bottom ovens (Tfield.h:113); 1 = oven surrounded (Tfield.h:224) */
    int sh_seed;             /* < 0: SH starts at zero; >= 0: seeded N(0, 1e-20) (Efields.h:129-144) */
    int device;              /* CUDA device ordinal */
    int crystal;             /* refractive index n(L, T): SHG_CRYSTAL_SPPLT (Crystal.h:55-71) or
                              * SHG_CRYSTAL_PPLN (README.md:48-49; see shg_index) */
} shg_config;

#define SHG_CRYSTAL_SPPLT 0  /* MgO:sPPLT, Bruner et al. Sellmeier: the reference's n(L, T) */
#define SHG_CRYSTAL_PPLN 1   /* PPLN: congruent LiNbO3, Jundt, Opt. Lett. 22, 1553 (1997) */

/* Fills `cfg` with the reference's compiled-in values (64x64x200 grid, 2000x1000x30000 um
 * MgO:sPPLT crystal, Crystal.h:26-53), thermal off, open-top BC, zero SH start, device 0. */
int shg_config_init(shg_config *cfg);

/* n(L, T) of Crystal.h:55-71 (extraordinary index at wavelength lambda_um [um] and
 * temperature temp_c [C]) for the crystal SHG_CRYSTAL_SPPLT (the reference's Bruner et al.
 * Sellmeier, bit-identical) or SHG_CRYSTAL_PPLN (periodically poled lithium niobate: the
 * temperature-dependent Sellmeier fit of congruent LiNbO3 by D. H. Jundt, Opt. Lett. 22,
 * 1553-1555 (1997); the reference's README names an MgO:PPLN crystal but its code has no
 * routine for it). Both are evaluated in double and rounded to float. */
int shg_index(int crystal, float lambda_um, float temp_c, float *n);

typedef struct shg_handle shg_handle;

/* Allocates the device state of one solve (the Efields/Tfield/PhaseMatching/Solver
 * objects of Solver.h:283-285 and 126-146). Grids must be square with NX = NY a power of
 * two in [16, 256]; other grids return SHG_ERR_UNSUPPORTED. */
int shg_create(const shg_config *cfg, shg_handle **out);
int shg_destroy(shg_handle *h);

/* Solver::run (Solver.h:279-355), same arguments in the same order. The output fields are
 * the state at the top of slice NZ-1 (what Solver::CWES saves as Pump_out/Signal_out,
 * Solver.h:250-255) and stay on the device until read. save_only_last / save_temperature
 * select the Files.h text outputs when an output directory is set (shg_set_output_dir). */
int shg_run(shg_handle *h, float power, float waist, float focalpoint, float temp, float t_inf,
            float t_peltier1, float t_peltier2, int save_only_last, int save_temperature);
/* Directory for the reference's text outputs (Files.h:19-79) written by shg_run: with
 * save_only_last, Pump_out_{r,i}.dat / Signal_out_{r,i}.dat (top of slice NZ-1); without it,
 * Pump_<s>_{r,i}.dat / Signal_<s>_{r,i}.dat for every slice s (Solver.h:250-262); with
 * save_temperature on a thermal handle, Tfinal_<z>.dat (Solver.h:340). NULL or "" turns
 * file output off (the default). */
int shg_set_output_dir(shg_handle *h, const char *dir);

/* Efields::setInputPump (Efields.h:174 -> setPump, Efields.h:74): Gaussian pump with the
 * refractive index taken at temperature tc. */
int shg_set_input_pump(shg_handle *h, float power, float focalpoint, float waist, float tc);
/* Arbitrary input fields (host, NX*NY complex each); sh may be NULL for a zero start. The
 * reference builds only the Gaussian of Efields.h:74-104 and the noise of Efields.h:129-144. */
int shg_set_input_fields(shg_handle *h, const float *pump, const float *sh);
/* Solver::CWES (Solver.h:245) without THERMAL from the current input fields, with the
 * propagators (Efields.h:186) and the constant phase mismatch (PhaseMatching.h:113)
 * set at temperature `temp`. */
int shg_cwes(shg_handle *h, float temp);
/* Solver::CWES (Solver.h:245) as above, with device pointers (NX*NY complex64 each) and a
 * cudaStream_t (NULL = default). */
int shg_cwes_device(shg_handle *h, float temp, const void *pump_in, const void *sh_in, void *pump_out,
                    void *sh_out, void *stream);

/* Results of the last run: the Pump_out / Signal_out state of Solver.h:250-255. Fields: host
 * buffers of NX*NY complex (interleaved float). */
int shg_get_fields(shg_handle *h, float *pump_out, float *sh_out);
/* P = 1/2 eps0 c n sum|A|^2 dx dy with n the pump / SH index at the run temperature, and the
 * efficiency P_SH(out) / P_pump(in) (the reference prints neither; its power normalisation
 * is that of setPump, Efields.h:88). */
int shg_get_powers(shg_handle *h, double *p_pump_in, double *p_sh_out, double *p_pump_out);
int shg_efficiency(shg_handle *h, double *eta);

const char *shg_last_error(void);

/* ---- Gradients (adjoint z-march, no counterpart in the reference) ---------------- */
/* Gradient of the output SH power L = 1/2 eps0 c n_s dx dy sum|S_out|^2 of the plain CWES
 * (shg_cwes_device semantics, fields at the top of slice NZ-1) with respect to the input
 * fields (grad_pump / grad_sh: device, NX*NY complex64, as dL/dRe + i dL/dIm; either may be
 * NULL), the oven temperature (input fields held fixed) and the poling period.
 * `checkpoints` states are kept in the forward pass (segments replayed backwards).
 * out4: [0] L (W), [1] dL/dT (W/K), [2] dL/dLambda (W/um), [3] dL/d(delta k) (W um).
 * Synchronises `stream`. */
int shg_grad_device(shg_handle *h, float temp, const void *pump_in, const void *sh_in, int checkpoints,
                    void *grad_pump, void *grad_sh, double *out4, void *stream);
/* Gradient of the SH output power of Solver::run's plain path (Solver.h:342-348): the input
 * pump is the focused Gaussian of setPump (Efields.h:74-104, index at `temp`) of (power,
 * waist, focalpoint), times pump_factor when given (device, NX*NY complex64, e.g. a seeded
 * perturbation; NULL: 1); the SH starts at zero; propagators and delta-k at `temp`.
 * grad_pump (device, may be NULL) receives dL/dA of the input pump A (dL/dRe + i dL/dIm).
 * out8: [0] L (W), [1] dL/dT with the input field held fixed (W/K), [2] dL/dLambda (W/um),
 * [3] dL/d(delta k) (W um), [4] dL/dfocalpoint (W/um), [5] dL/dwaist (W/um), [6] dL/dPower
 * (W/W), [7] dL/dT including the pump's index n_p(T) (W/K). The pump-parameter terms are
 * FP64 sums of the adjoint field against the analytic derivatives of setPump. Synchronises
 * `stream`. */
int shg_grad_run(shg_handle *h, float power, float waist, float focalpoint, float temp, const void *pump_factor,
                 int checkpoints, void *grad_pump, double *out8, void *stream);
/* Changes the poling period (Crystal.h:43) of a plain handle for the following runs. */
int shg_set_poling_period(shg_handle *h, float lambda_qpm);

/* ---- THERMAL (cfg.thermal = 1) ----------------------------------------------------- */
/* After shg_run on a thermal handle: the final temperature tensor (NX*NY*NZ floats,
 * Tfield::Tfinal) and the Jacobi sweep count of each of the five outer iterations of
 * Solver.h:295-338 (-1 for iterations not run). */
int shg_get_temperature(shg_handle *h, float *T);
int shg_get_jacobi_counts(shg_handle *h, int *counts5);
/* Jacobi stop rule of a THERMAL handle: rel_tol <= 0 (default) is the reference's rule
 * (Solver.h:302-324: residual checked at sweep 0 and every 5000); rel_tol > 0 stops once
 * ||T_k+1 - T_k|| / ||T_k+1|| < rel_tol (checked every check_every sweeps, at most
 * max_sweeps per Jacobi solve), the relative-residual mode of the THERMAL workload.
 * shg_get_jacobi_residual gives the last relative residual checked (-1 if none). */
int shg_set_jacobi_rule(shg_handle *h, double rel_tol, int check_every, int max_sweeps);
int shg_get_jacobi_residual(shg_handle *h, double *rel);
/* Components on host buffers (NX = NY; grid from cfg): Tfield.h:31-110 initial
 * temperature; `nsweeps` sweeps of Tfield.h:113 (bc 0) or Tfield.h:224 (bc 1), each followed
 * by Tinic <- Tfinal (Solver.h:321), T updated in place, Q the heat source; and
 * PhaseMatching.h:41-54 delta-k(T) with the two refractive indices (any output may be NULL). */
int shg_init_temperature(const shg_config *cfg, float temp, float t1, float t2, int bc, float *T_out);
int shg_heat_sweeps(const shg_config *cfg, float *T_inout, const float *Q, float t_inf, int nsweeps, int bc);
int shg_dk_thermal(const shg_config *cfg, const float *T, float *DK, float *NP, float *NS);
/* `nsweeps` heat sweeps (Tfield.h:113 / Tfield.h:224) on device buffers: Ta holds T on entry, Tb an identical copy (the
 * voxels the stencil never writes must match); sweep k writes the other buffer, so the
 * result is in Ta for even nsweeps and in Tb for odd. QK = Q / k_th per voxel. */
int shg_heat_sweeps_device(const shg_config *cfg, void *Ta, void *Tb, const void *QK, float t_inf, int nsweeps, int bc,
                           void *stream);

/* ---- Batched sweep: many independent plain solves in one device schedule ----------- */
/* Replaces SHG.sh:73-101, which runs one ./SHG process per sweep point (SHG.sh:81). */
typedef struct shg_instance {
    int nx, ny, nz;          /* per-solve grid (square, power of two) */
    float lx, ly;            /* per-solve window */
    float power, waist, temp, focal;  /* Solver::run arguments (Temp also sets delta-k) */
} shg_instance;

typedef struct shg_batch shg_batch;
/* `crystal` supplies lz, lp, deff, lambda_qpm, absorption and walk-off; its grid and
 * window fields are ignored. */
int shg_batch_create(const shg_config *crystal, const shg_instance *inst, int n, shg_batch **out);
int shg_batch_destroy(shg_batch *b);
/* Runs every solve and copies the efficiencies (n doubles) to the host; when sh_out_all
 * is not NULL it receives the SH output fields of all solves back to back in solve order
 * (solve i at the complex offset given by shg_batch_field_offsets). A batch whose device
 * memory exceeds the free memory returns SHG_ERR_NOMEM from shg_batch_create (checked on
 * the host before allocating). When a solve's efficiency is NaN or infinite (e.g. a NaN
 * parameter), every value is still stored and SHG_ERR_NONFINITE names the first such
 * solve (also from shg_batch_results). */
int shg_batch_run(shg_batch *b, double *eta, float *sh_out_all);
/* After a run: output pump and SH fields of all solves (same layout as sh_out_all above);
 * either pointer may be NULL. */
int shg_batch_fields(shg_batch *b, float *pump_out_all, float *sh_out_all);
/* Replaces the run parameters of every solve (grids must stay the same); the next run
 * uploads them. */
int shg_batch_set_instances(shg_batch *b, const shg_instance *inst, int n);
/* offsets[0..n]: complex offset of each solve's field in the contiguous output; offsets[n]
 * is the total. */
int shg_batch_field_offsets(shg_batch *b, long long *offsets);
/* Device-only run on `stream` (results stay on the device); shg_batch_results copies the
 * efficiencies after the stream has been synchronised. */
int shg_batch_run_async(shg_batch *b, void *stream);
int shg_batch_results(shg_batch *b, double *eta);
/* Bytes one re-parameterised run moves: parameters and device descriptors uploaded,
 * and the SH output fields of all solves. */
int shg_batch_io_bytes(shg_batch *b, long long *h2d_per_run, long long *d2h_fields);
/* Number of kernel launches one run issues. */
int shg_batch_launch_count(shg_batch *b, int *launches);

/* Schedule autotuner. Each grid-size class of the batch marches either as streaming
 * row/column launches or as one persistent resident launch (a thread-block cluster per
 * solve, fields in shared memory) in one of several (cluster size, CTAs per SM) variants.
 * Resident variants also differ in the line-FFT split (n = 64: 8 x 8 or 16 x 4 points).
 * Unless the environment variable SHG_MARCH is "streaming", "resident" (default variants)
 * or lists a schedule per grid ("64:1/1,128:4/2,256:16/2", "64:1/1/4", "64:streaming",
 * "128:coop"), the first run times every candidate on the class's own solves and keeps the
 * fastest (cached per device and class shape for the process). A batch of one solve has one
 * more candidate, "coop": the whole march in one cooperative launch (row and column passes
 * of the streaming kernels, bit-identical, separated by grid-wide barriers whose waits are
 * bounded; a wait that gives up makes the run's result calls return SHG_ERR_CUDA). shg_batch_autotune does that now, outside any
 * stream capture; shg_batch_schedule writes the choices and trial times as text. */
int shg_batch_autotune(shg_batch *b, void *stream);
/* Fixes the schedule of the class with grid n: resident = 0 streaming, resident = 2 the
 * persistent cooperative grid (a batch of one solve only; cluster_size and ctas_per_sm
 * unused), resident = 3 the cluster march (n in {64, 128, 256}: each solve in one cluster
 * of 8 / 16 / 16 CTAs of 512 threads, one thread per point in the pointwise phase;
 * cluster_size and ctas_per_sm unused), else the resident variant with cluster_size CTAs per cluster and ctas_per_sm
 * CTAs per SM (variants: n <= 32 (1, 1); n = 64 (1, 1), (1, 2), (2, 2), (2, 4); n = 128
 * (2, 1), (4, 1), (4, 2); n = 256 (8, 1), (16, 1), (16, 2)). SHG_ERR_UNSUPPORTED if the
 * variant does not exist or fit. */
int shg_batch_set_schedule(shg_batch *b, int n, int resident, int cluster_size, int ctas_per_sm);
/* Same for a resident variant with a given line-FFT split: threads_per_line G, each thread
 * holding N/G points (n = 64: G = 8 or 4; other grids: their one split). */
int shg_batch_set_schedule_split(shg_batch *b, int n, int cluster_size, int ctas_per_sm, int threads_per_line);
int shg_batch_schedule(shg_batch *b, char *buf, int len);
/* Diagnostic: one concurrent run without a graph, with events around each grid-size class
 * launched on its own stream as a run launches them; start_end[2k], start_end[2k+1] = start
 * and end of class k (ascending grid order) in ms after the common start. */
int shg_batch_timeline(shg_batch *b, double *start_end, int max_classes, int *n_classes, void *stream);

/* Per-kernel timing of one un-captured run: CUDA events around every launch, summed per
 * kernel (name like "rows<128>"), with the algorithmic bytes those launches must move
 * (fields read and written once; propagators read once in the column pass). */
typedef struct shg_kernel_stat {
    char name[32];
    int launches;
    double ms;
    double bytes;
} shg_kernel_stat;
int shg_batch_profile(shg_batch *b, shg_kernel_stat *stats, int max_stats, int *n_stats);

/* ---- Plain CWES without device allocation ---------------------------------------- */
/* No counterpart in the reference. For callers that cannot call cudaMalloc (device memory
 * owned up front by another allocator, allocation-free real-time loops, plugin hosts that
 * forbid device allocation): the same plain CWES as shg_cwes_device, with every working
 * buffer in one fixed file-scope device array instead of allocated memory. cfg gives the
 * grid and crystal (NX = NY a power of two in [16, 128], NZ in [2, 4096]; larger sizes
 * return SHG_ERR_INVALID); pump_in / sh_in (NULL: zero SH start) / pump_out / sh_out are
 * caller-owned device buffers of NX*NY complex64; when eta is not NULL the call
 * synchronises `stream` and stores the efficiency. The first call on a device, with that
 * device current, does a one-time set-up (array address, twiddle tables); make it before
 * any stream capture. That set-up is cached per device ordinal for the process, so a
 * device reset after the first call is not supported. All calls share the array and it
 * keeps the last call's contents: calls that overlap on the GPU race. */
int shg_cwes_noalloc(const shg_config *cfg, float temp, const void *pump_in, const void *sh_in,
                     void *pump_out, void *sh_out, double *eta, void *stream);

/* ---- Check build (no counterpart in the reference) ----------------------------------- */
/* *enabled = 1 in the library built with device-side index checks (build.py variant
 * "check": descriptors, stages, field / propagator / slice / voxel indices, cluster ranks,
 * TMA box coordinates), else 0. A failed check never traps: it records its site and value
 * and skips the access. This call synchronises the device, then reads and clears the first
 * failure of every kernel translation unit: *site = 0 for none, else the check site
 * (kChk* in csrc/shg_check.cuh), *value the offending index or value. */
int shg_check_status(int *enabled, int *site, long long *value);
/* Check build only: a kernel that touches no memory records (site 1, value), showing that a
 * failure reaches shg_check_status. SHG_ERR_UNSUPPORTED in other builds. */
int shg_check_selftest(long long value);

/* ---- Batched gradient of the THERMAL z-march (fixed temperature fields) ----------- */
/* No counterpart in the reference (its THERMAL Solver::run, Solver.h:287-340, is forward
 * only). `count` solves on one grid (cfg: NX = NY a power of two in [16, 256]; the
 * crystal and heat constants as for a THERMAL handle), each with its own temperature field
 * held fixed. Solve i's loss is its SH output power (the state at the top of slice NZ-1 of
 * the THERMAL CWES, Solver.h:245-276, without heat-source updates); the gradient is taken
 * with respect to its input pump, in the form dL/dRe + i dL/dIm. Propagators, the Gaussian
 * reference pump and the power convention use n at T[NX/2, NY/2, 0] (Efields.h:77,110). */
typedef struct shg_thgrad shg_thgrad;
int shg_thgrad_create(const shg_config *cfg, int count, shg_thgrad **out);
void shg_thgrad_destroy(shg_thgrad *b);
/* Solver::run (THERMAL) for solve i with a Gaussian pump (Solver::run's arguments); its
 * final temperature field is kept, and that pump becomes the solve's reference input.
 * counts (5 ints, may be NULL) receives the Jacobi sweeps of each outer iteration. */
int shg_thgrad_solve_temperature(shg_thgrad *b, int i, float power, float waist, float focal, float temp,
                                 float t_inf, float t1, float t2, int *counts);
/* Solve i's temperature field given directly (host, NX*NY*NZ floats, IDX(x,y,z)) and the
 * Gaussian reference input of (power, waist, focal). */
int shg_thgrad_set_temperature(shg_thgrad *b, int i, const float *T, float power, float waist, float focal);
int shg_thgrad_get_temperature(shg_thgrad *b, int i, float *T);
/* The solves' Gaussian reference inputs into a device buffer of count*NX*NY complex64. */
int shg_thgrad_gaussian_pumps(shg_thgrad *b, void *pump, void *stream);
/* Forward pass of every solve: pump_in (device, count*NX*NY complex64, solve-major), SH
 * start zero; pump_out / sh_out (device, may be NULL) receive the output fields; p_sh /
 * p_in (host, count doubles, may be NULL; the call then synchronises `stream`) the SH
 * output power and the input pump power [W]. */
int shg_thgrad_forward(shg_thgrad *b, const void *pump_in, void *pump_out, void *sh_out, double *p_sh, double *p_in,
                       void *stream);
/* Forward and reverse pass: grad_pump (device, count*NX*NY) = dP_SH,i / dA_in,i.
 * checkpoints < NZ-1 keeps that many states per solve and replays segments; checkpoints
 * >= NZ-1 keeps every step (no replay; 2*(NZ-1) states per solve). */
int shg_thgrad_gradient(shg_thgrad *b, const void *pump_in, int checkpoints, void *grad_pump, double *p_sh,
                        double *p_in, void *stream);
/* Kernel launches of the last forward or gradient pass; device memory held. */
int shg_thgrad_launch_count(const shg_thgrad *b);
double shg_thgrad_device_bytes(const shg_thgrad *b);

/* ---- Components, for tests ------------------------------------------------------- */
/* Unnormalised 2D DFT of an n x n complex array on the device (sign -1 forward, +1
 * backward, FFTW's convention; the fftwf plans of Solver::diffraction, Solver.h:156-190), device pointers, in place allowed. */
int shg_dft2d_device(int n, int sign, const void *in, void *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif
