// ORACLE — test infrastructure only. Implements the fftw3.h stand-in beside it with the
// DFT restatement in ../dft_ref.h (float working precision, double-evaluated twiddles).
#include "fftw3.h"

#include "../dft_ref.h"

struct oracle_fftwf_plan_s {
    int n0, n1, sign;
    float *in, *out;
};

extern "C" fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out,
                                        int sign, unsigned flags) {
    (void)flags;
    auto *p = new oracle_fftwf_plan_s;
    p->n0 = n0;
    p->n1 = n1;
    p->sign = sign;
    p->in = reinterpret_cast<float *>(in);
    p->out = reinterpret_cast<float *>(out);
    // Tables are built at planning time, as FFTW does.
    dftref::line_tables<float>(n0);
    dftref::line_tables<float>(n1);
    return p;
}

extern "C" void fftwf_execute(const fftwf_plan p) {
    dftref::dft2d<float>(p->in, p->out, p->n0, p->n1, p->sign);
}

extern "C" void fftwf_destroy_plan(fftwf_plan p) { delete p; }
