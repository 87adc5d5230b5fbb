// ORACLE — test infrastructure only. Built by oracle/build_ref.py into oracle/_ref/
// (git-ignored); nothing in the product links it.
//
// Compiles the reference's own headers where they lie (src/headers/*.h of
// alfredos84/SHG_Focused_Gaussian_Beams, included unmodified through -I) into one
// translation unit, the way src/SHG.cpp:4-22 does, but with the grid and crystal
// constants supplied by this file so that one recipe builds every configuration:
//
//   * NX, NY, NZ, TSIZE and the byte counts are defined here exactly as SHG.cpp:11-20
//     defines them (values from -DREF_NX/-DREF_NY/-DREF_NZ).
//   * The crystal constants that the configurations change (Crystal.h:31-53: LX, LY, LZ,
//     dx, dy, dz, deff, dQ, Lambda, alpha_crp, alpha_crs, beta_crs, rhop, rhos,
//     thermal_cond, heat_trf_coeff) are renamed by the preprocessor while Crystal.h is
//     read, so its own definitions become unused `ref_default_*` constants, and are then
//     redefined below with the same formulas (dx = LX/(NX-1) etc., Crystal.h:34-36,42).
//   * The FFTW calls resolve to oracle/fftw_shim (FFTW is not installed here).
//
// Exported C entry points wrap the reference's functions one by one so that tests can
// compare the oracle restatement (oracle/shg_oracle.cpp) and the CUDA library against
// them; `ref_main` is SHG.cpp's main (argv P waist T1 T2 SOLS STMP -> Solver::run).
#include "headers/Libraries.h"

using real_t = float;
using complex_t = std::complex<real_t>;

const uint NX = REF_NX;
const uint NY = REF_NY;
const uint NZ = REF_NZ;
const uint NXY = NX * NY;
const uint TSIZE = NX * NY * NZ;
const size_t nBytes2Dr = sizeof(real_t) * NXY;
const size_t nBytes2Dc = sizeof(complex_t) * NXY;
const size_t nBytes3Dr = sizeof(real_t) * TSIZE;

#define LX ref_default_LX
#define LY ref_default_LY
#define LZ ref_default_LZ
#define dx ref_default_dx
#define dy ref_default_dy
#define dz ref_default_dz
#define deff ref_default_deff
#define dQ ref_default_dQ
#define Lambda ref_default_Lambda
#define alpha_crp ref_default_alpha_crp
#define alpha_crs ref_default_alpha_crs
#define beta_crs ref_default_beta_crs
#define rhop ref_default_rhop
#define rhos ref_default_rhos
#define thermal_cond ref_default_thermal_cond
#define heat_trf_coeff ref_default_heat_trf_coeff

#include "headers/Common.h"
#include "headers/Operators.h"
#include "headers/Files.h"
#include "headers/Crystal.h"

#undef LX
#undef LY
#undef LZ
#undef dx
#undef dy
#undef dz
#undef deff
#undef dQ
#undef Lambda
#undef alpha_crp
#undef alpha_crs
#undef beta_crs
#undef rhop
#undef rhos
#undef thermal_cond
#undef heat_trf_coeff

const real_t LX = REF_LX;
const real_t LY = REF_LY;
const real_t LZ = REF_LZ;
const real_t dx = LX / (NX - 1);
const real_t dy = LY / (NY - 1);
const real_t dz = LZ / (NZ - 1);
const real_t deff = REF_DEFF;
const real_t dQ = (2.0 / PI) * deff;
const real_t Lambda = REF_LAMBDA;
const real_t alpha_crp = REF_ALPHA_P;
const real_t alpha_crs = REF_ALPHA_S;
const real_t beta_crs = REF_BETA_S;
const real_t rhop = REF_RHO_P;
const real_t rhos = REF_RHO_S;
const real_t thermal_cond = REF_KTH;
const real_t heat_trf_coeff = REF_HTC;

#include "headers/Efields.h"
#include "headers/Tfield.h"
#include "headers/PhaseMatching.h"
#include "headers/Solver.h"

#include <cstring>

namespace {
std::vector<real_t> uniform_T(real_t Tc) { return std::vector<real_t>((size_t)TSIZE, Tc); }
}  // namespace

extern "C" {

int ref_is_thermal(void) {
#ifdef THERMAL
    return 1;
#else
    return 0;
#endif
}

void ref_grid(int *nx, int *ny, int *nz) {
    *nx = (int)NX;
    *ny = (int)NY;
    *nz = (int)NZ;
}

// dx, dy, dz, dQ, deff, Lambda, alpha_p, alpha_s, beta_s, LX, LY, LZ
void ref_constants(float *o) {
    o[0] = dx; o[1] = dy; o[2] = dz; o[3] = dQ; o[4] = deff; o[5] = Lambda;
    o[6] = alpha_crp; o[7] = alpha_crs; o[8] = beta_crs; o[9] = LX; o[10] = LY; o[11] = LZ;
}

// Crystal.h:116
float ref_n(float L, float T) { return n(L, T); }

// Efields.h:74 (Temp at the grid centre of slice 0, as setPump reads it)
void ref_set_pump(float *pump, float Power, float focalpoint, float waist, float Tc) {
    auto T = uniform_T(Tc);
    setPump(reinterpret_cast<complex_t *>(pump), Power, focalpoint, waist, T.data());
}

// Efields.h:129 with the clock seed replaced by `seed` (same engine and distribution).
void ref_noise(float *sh, unsigned seed) {
    std::default_random_engine generator(seed);
    std::normal_distribution<real_t> distribution(0.0, 1.0e-20);
    for (uint i = 0; i < NX * NY; ++i) {
        real_t a1 = distribution(generator);
        real_t a2 = distribution(generator);
        sh[2 * i] = a1;
        sh[2 * i + 1] = a2;
    }
}

// Efields.h:186-192: beamPropagator then fftShift2D on both propagators.
void ref_propagators(float *hp, float *hs, float Tc) {
    auto T = uniform_T(Tc);
    complex_t *p = reinterpret_cast<complex_t *>(hp), *s = reinterpret_cast<complex_t *>(hs);
    beamPropagator(p, s, T.data());
    fftShift2D(p);
    fftShift2D(s);
}

// PhaseMatching.h:57 (one value of the constant table)
float ref_dk_constant(float Temp) {
    std::vector<real_t> DK((size_t)TSIZE);
    initDKConstant(DK.data(), Temp);
    return DK[0];
}

// Solver.h:156 on a pair of fields (the Efields propagators are set from Tc first).
void ref_diffraction(float *pump, float *sh, float Tc) {
    Efields *A = new Efields;
    auto T = uniform_T(Tc);
    A->setPropagators(T.data());
    std::memcpy(A->Pump, pump, nBytes2Dc);
    std::memcpy(A->Signal, sh, nBytes2Dc);
    Solver S;
    S.diffraction(A);
    std::memcpy(pump, A->Pump, nBytes2Dc);
    std::memcpy(sh, A->Signal, nBytes2Dc);
    delete A;
}

// Solver.h:245 CWES loop (no THERMAL), fields given; returns the state saved at the top
// of slice NZ-1 (what CWES writes as Pump_out/Signal_out) and the state after NZ steps.
void ref_cwes_plain(const float *pump_in, const float *sh_in, float Temp, float *pump_out,
                    float *sh_out, float *pump_end, float *sh_end) {
#ifdef THERMAL
    (void)pump_in; (void)sh_in; (void)Temp; (void)pump_out; (void)sh_out; (void)pump_end; (void)sh_end;
#else
    Efields *A = new Efields;
    Tfield *T = new Tfield;
    PhaseMatching *DK = new PhaseMatching;
    T->setTemperature(Temp);
    std::memcpy(A->Pump, pump_in, nBytes2Dc);
    std::memcpy(A->Signal, sh_in, nBytes2Dc);
    A->setPropagators(T->Tfinal);
    DK->setInicialDKConstant(Temp);
    Solver S;
    real_t z = 0.0;
    for (uint s = 0; s < NZ; ++s) {
        if (s == NZ - 1) {
            std::memcpy(pump_out, A->Pump, nBytes2Dc);
            std::memcpy(sh_out, A->Signal, nBytes2Dc);
        }
        S.SSFM(A, T, DK, Temp, z, s);
        z += dz;
    }
    if (pump_end) std::memcpy(pump_end, A->Pump, nBytes2Dc);
    if (sh_end) std::memcpy(sh_end, A->Signal, nBytes2Dc);
    delete A;
    delete T;
    delete DK;
#endif
}

// Tfield.h:31,48,71 initial temperature tensors.
void ref_init_temperature(float *T, float Temp, float T1, float T2, int bc) {
    initTemperature(T, Temp);
    if (bc == 0)
        initBottomOvensTemperature(T, T1, T2);
    else
        initOvenSurrounded(T, T1, T2);
}

// `nsweeps` Jacobi sweeps of Tfield.h:113 (bc 0) or Tfield.h:224 (bc 1), with the copy
// Tinic <- Tfinal after each sweep (Solver.h:321). T is updated in place.
void ref_heat_sweeps(float *T, const float *Q, float T_inf, int nsweeps, int bc) {
    std::vector<real_t> Tf(T, T + TSIZE), Ti(T, T + TSIZE), Qv(Q, Q + TSIZE);
    for (int k = 0; k < nsweeps; ++k) {
        if (bc == 0)
            heatEquationTopOpen(Tf.data(), Ti.data(), T_inf, Qv.data());
        else
            kernelHeatEquationOvenSurrounded(Tf.data(), Ti.data(), T_inf, Qv.data());
        copyTensor<real_t>(Ti.data(), Tf.data());
    }
    std::memcpy(T, Tf.data(), nBytes3Dr);
}

// Tfield.h:13
float ref_reduced_sum(const float *Tf, const float *Ti) {
    return reducedSum(const_cast<real_t *>(Tf), const_cast<real_t *>(Ti));
}

// PhaseMatching.h:41
void ref_dk_thermal(float *DK, const float *T) { setInicialDKThermal(DK, const_cast<real_t *>(T)); }

// Tfield.h:277
void ref_set_q(float *Q, const float *T, const float *pump, const float *sh, int s) {
    setQ(Q, const_cast<real_t *>(T), reinterpret_cast<complex_t *>(const_cast<float *>(pump)),
         reinterpret_cast<complex_t *>(const_cast<float *>(sh)), (uint)s);
}

// Solver::run's THERMAL branch (Solver.h:287-340) driven through the same calls, with
// the SH start fixed (zeros or seeded noise) instead of clock-seeded noise, a choice of
// boundary mode, and binary outputs: the fields saved at the top of slice NZ-1 of the
// last CWES, the final temperature tensor, and the Jacobi sweep count of every outer
// iteration (counts[0..4], -1 when not run). Returns the number of outer iterations run.
int ref_thermal_run(float Power, float waist, float focalpoint, float Temp, float T_inf,
                    float T1, float T2, int bc, int sh_seed, float *pump_out, float *sh_out,
                    float *T_out, int *counts) {
#ifndef THERMAL
    (void)Power; (void)waist; (void)focalpoint; (void)Temp; (void)T_inf; (void)T1; (void)T2;
    (void)bc; (void)sh_seed; (void)pump_out; (void)sh_out; (void)T_out; (void)counts;
    return -1;
#else
    Efields *A = new Efields;
    Tfield *T = new Tfield;
    PhaseMatching *DK = new PhaseMatching;
    Solver S;
    T->setTemperature(Temp);
    if (bc == 0)
        T->setBottomOvens(T1, T2);
    else
        T->setOvenSurrounded(T1, T2);
    T->setInitialQ();
    for (int i = 0; i < 5; ++i) counts[i] = -1;
    uint global_count = 0, num_of_iter = 5;
    int outer = 0;
    while (global_count < num_of_iter) {
        real_t tol = 5e-4 / TSIZE;
        real_t Reduced_sum = 1.0, aux_sum = -1.0f;
        uint counter_T = 0;
        while (Reduced_sum >= tol) {
            if (bc == 0)
                T->upDate(T_inf);
            else
                kernelHeatEquationOvenSurrounded(T->Tfinal, T->Tinic, T_inf, T->Q);
            uint chkconv = 5000;
            if (counter_T % chkconv == 0) {
                if (counter_T > 0) aux_sum = Reduced_sum;
                Reduced_sum = T->checkConvergence();
                if (Reduced_sum == aux_sum) Reduced_sum = 0.5 * tol;
            }
            copyTensor<real_t>(T->Tinic, T->Tfinal);
            counter_T++;
        }
        counts[outer++] = (int)counter_T;
        DK->setDKFromTemperature(T);
        A->setInputPump(Power, focalpoint, waist, T->Tfinal);
        if (sh_seed < 0)
            std::memset((void *)A->Signal, 0, nBytes2Dc);
        else
            ref_noise(reinterpret_cast<float *>(A->Signal), (unsigned)sh_seed);
        A->setPropagators(T->Tfinal);
        // CWES (Solver.h:245-276) with the slice-(NZ-1) save captured in memory.
        real_t z = 0.0;
        for (uint s = 0; s < NZ; ++s) {
            if (s == NZ - 1) {
                std::memcpy(pump_out, A->Pump, nBytes2Dc);
                std::memcpy(sh_out, A->Signal, nBytes2Dc);
            }
            S.SSFM(A, T, DK, Temp, z, s);
            T->upDateQ(A, s);
            z += dz;
        }
        if (counter_T == 1 and global_count != 0) global_count = num_of_iter;
        global_count++;
    }
    std::memcpy(T_out, T->Tfinal, nBytes3Dr);
    delete A;
    delete T;
    delete DK;
    return outer;
#endif
}

// src/SHG.cpp:24-102: argv = P waist T1 T2 SOLS STMP; focal point LZ/2, T_inf 25.
int ref_main(int argc, char **argv) {
    if (argc < 7) return 2;
    real_t Power = atof(argv[1]);
    real_t waist = atof(argv[2]);
    real_t focalpoint = 0.5 * LZ;
    real_t Temp = atof(argv[3]);
    real_t T_inf = 25;
    real_t Tpeltier1 = atof(argv[3]);
    real_t Tpeltier2 = atof(argv[4]);
    bool save_only_last = atoi(argv[5]);
    bool save_temperature = atoi(argv[6]);
    double iStart = seconds();
    Solver *solver = new Solver;
    solver->run(Power, waist, focalpoint, Temp, T_inf, Tpeltier1, Tpeltier2, save_only_last,
                save_temperature);
    delete solver;
    double iElaps = seconds() - iStart;
    std::cout << "ref_main elapsed " << std::setprecision(9) << iElaps << " s" << std::endl;
    return 0;
}

}  // extern "C"

#ifdef ORACLE_REF_MAIN
int main(int argc, char **argv) { return ref_main(argc, argv); }
#endif
