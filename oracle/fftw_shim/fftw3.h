/* ORACLE — test infrastructure only.
 *
 * Stand-in for the subset of the FFTW3 single-precision API that the reference calls
 * (Solver.h:161-187: fftwf_plan_dft_2d, fftwf_execute, fftwf_destroy_plan; constants
 * FFTW_FORWARD, FFTW_BACKWARD, FFTW_ESTIMATE; type fftwf_complex). FFTW itself is not
 * installed here and the reference does not vendor or pin it. The transform follows
 * FFTW's published definition (unnormalised, row-major n0 x n1, exp(sign*2*pi*i*jk/n));
 * the implementation is dft_ref.h. Only the reference build under oracle/_ref links it.
 */
#ifndef ORACLE_FFTW_SHIM_FFTW3_H
#define ORACLE_FFTW_SHIM_FFTW3_H

#ifdef __cplusplus
extern "C" {
#endif

typedef float fftwf_complex[2];
typedef struct oracle_fftwf_plan_s *fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out,
                             int sign, unsigned flags);
void fftwf_execute(const fftwf_plan plan);
void fftwf_destroy_plan(fftwf_plan plan);

#ifdef __cplusplus
}
#endif

#endif
