// `shg` command line: the argument list of the reference's SHG binary
// (src/SHG.cpp:37-50, driven by src/SHG.sh:81):
//
//     shg <P [W]> <waist [um]> <T1 [C], also Temp> <T2 [C]> <SOLS 0/1> <STMP 0/1> [options]
//
// The grid and crystal, compile-time constants in the reference (SHG.cpp:11-13,
// Crystal.h:26-53), are options here: --nx N --ny N --nz N --lx um --ly um --lz um
// --deff um/V --lambda um --alpha-p 1/um --alpha-s 1/um --beta-s um/W --thermal --bc 0|1
// --crystal spplt|ppln --outdir DIR --device K. Output files follow Files.h:36-57
// (Pump_out_r.dat, ...); the screen output and the CPUTime_NZ_<NZ>_N_<NX>_T.txt timing file
// follow SHG.cpp:52-97.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/shg.h"

namespace {

int fail(const char *what, int rc) {
    std::cerr << what << " failed (" << rc << "): " << shg_last_error() << std::endl;
    return 1;
}

// The crystal block of the parameter printout (Crystal.h:74-89), from the run-time config.
void print_crystal(const shg_config &c) {
    const float dx = c.lx / (c.nx - 1), dy = c.ly / (c.ny - 1), dz = c.lz / (c.nz - 1);
    std::cout << "\n\nCrystal properties:\n" << std::endl;
    std::cout << "Crystal dimensions = ( " << c.lx * 1e-3 << ", " << c.ly * 1e-3 << ", " << c.lz * 1e-3 << " ) mm"
              << std::endl;
    std::cout << "Crystal discretization (dz, dy, dz) = ( " << dx << ", " << dy << ", " << dz << " ) μm " << std::endl;
    std::cout << "Nonlinear crystal = " << (c.crystal == SHG_CRYSTAL_PPLN ? "PPLN" : "MgO:sPPLT") << std::endl;
    std::cout << "Eff. second-order susc., deff = " << c.deff << " μm/V" << std::endl;
    std::cout << "Grating period for QPM, Λ = " << c.lambda_qpm << " μm" << std::endl;
    std::cout << "Pump linear absorp., αp = " << c.alpha_p << " 1/μm" << std::endl;
    std::cout << "Signal linear absorp., αs = " << c.alpha_s << " 1/μm" << std::endl;
    std::cout << "Signal 2-photons absorp., βs = " << c.beta_s << " 1/μm" << std::endl;
    std::cout << "Pump walk-off angle, ρ = " << c.rho_p << " rad" << std::endl;
    std::cout << "Signal walk-off angle, ρ = " << c.rho_s << " rad" << std::endl;
    std::cout << "Thermal conductivity, k = " << c.kth << " W/μm K" << std::endl;
    std::cout << "Heat Transfer Coefficient, h = " << c.htc << " W/μm² K\n\n" << std::endl;
}

// Elapsed time in seconds, minutes or hours (Common.h:17-24).
void print_elapsed(double s) {
    if (s < 60.0)
        std::cout << "\n\n...time elapsed " << s << " seconds\n\n " << std::endl;
    else if (s < 3600.0)
        std::cout << "\n\n...time elapsed " << s / 60 << " minutes\n\n " << std::endl;
    else
        std::cout << "\n\n...time elapsed " << s / 3600 << " hours\n\n " << std::endl;
}

}  // namespace

int main(int argc, char **argv) {
    std::cout << "#######---SHG efficiency calculator (GB300)---#######\n\n" << std::endl;
    if (argc < 7) {
        std::cerr << "usage: shg P waist T1 T2 SOLS STMP [--nx N --ny N --nz N --lx um --ly um --lz um "
                     "--deff um/V --lambda um --alpha-p v --alpha-s v --beta-s v --thermal --bc 0|1 "
                     "--crystal spplt|ppln --outdir DIR --device K]"
                  << std::endl;
        return 2;
    }
    const auto t0 = std::chrono::steady_clock::now();
    shg_config cfg;
    shg_config_init(&cfg);
    std::string outdir = ".";
    for (int i = 7; i < argc; ++i) {
        const std::string a = argv[i];
        auto val = [&]() -> const char * {
            if (i + 1 >= argc) {
                std::cerr << "missing value for " << a << std::endl;
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "--nx") cfg.nx = std::atoi(val());
        else if (a == "--ny") cfg.ny = std::atoi(val());
        else if (a == "--nz") cfg.nz = std::atoi(val());
        else if (a == "--lx") cfg.lx = (float)std::atof(val());
        else if (a == "--ly") cfg.ly = (float)std::atof(val());
        else if (a == "--lz") cfg.lz = (float)std::atof(val());
        else if (a == "--deff") cfg.deff = (float)std::atof(val());
        else if (a == "--lambda") cfg.lambda_qpm = (float)std::atof(val());
        else if (a == "--alpha-p") cfg.alpha_p = (float)std::atof(val());
        else if (a == "--alpha-s") cfg.alpha_s = (float)std::atof(val());
        else if (a == "--beta-s") cfg.beta_s = (float)std::atof(val());
        else if (a == "--thermal") cfg.thermal = 1;
        else if (a == "--bc") cfg.bc = std::atoi(val());
        else if (a == "--crystal") {
            const std::string v = val();
            if (v == "spplt") cfg.crystal = SHG_CRYSTAL_SPPLT;
            else if (v == "ppln") cfg.crystal = SHG_CRYSTAL_PPLN;
            else {
                std::cerr << "unknown crystal " << v << " (spplt or ppln)" << std::endl;
                return 2;
            }
        }
        else if (a == "--outdir") outdir = val();
        else if (a == "--device") cfg.device = std::atoi(val());
        else {
            std::cerr << "unknown option " << a << std::endl;
            return 2;
        }
    }
    // SHG.cpp:37-50
    const float Power = (float)std::atof(argv[1]);
    const float waist = (float)std::atof(argv[2]);
    const float focalpoint = (float)(0.5 * cfg.lz);
    const float Temp = (float)std::atof(argv[3]);
    const float T_inf = 25;
    const float Tpeltier1 = (float)std::atof(argv[3]);
    const float Tpeltier2 = (float)std::atof(argv[4]);
    const bool save_only_last = std::atoi(argv[5]);
    const bool save_temperature = std::atoi(argv[6]);
    std::cout << "\n\nPump power =  " << Power << " W" << std::endl;
    std::cout << "Beam waist = " << waist << " μm" << std::endl;
    std::cout << "Focal distance = " << focalpoint << " μm" << std::endl;
    std::cout << "Phase-matching temperature =  " << Temp << " ºC" << std::endl;
    std::cout << "Environment temperature =  " << T_inf << " ºC" << std::endl;
    std::cout << "Peltier 1 temperature =  " << Tpeltier1 << " ºC" << std::endl;
    std::cout << "Peltier 2 temperature =  " << Tpeltier2 << " ºC\n" << std::endl;
    print_crystal(cfg);

    shg_handle *h = nullptr;
    int rc = shg_create(&cfg, &h);
    if (rc) return fail("shg_create", rc);
    rc = shg_set_output_dir(h, outdir.c_str());
    if (rc) return fail("shg_set_output_dir", rc);
    // Solver.h:250-262 / 340: Pump_out/Signal_out (SOLS=1) or every slice (SOLS=0), Tfinal (STMP=1)
    rc = shg_run(h, Power, waist, focalpoint, Temp, T_inf, Tpeltier1, Tpeltier2, save_only_last, save_temperature);
    if (rc) return fail("shg_run", rc);
    if (cfg.thermal) {
        int counts[5];
        if (shg_get_jacobi_counts(h, counts) == SHG_OK)
            for (int i = 0; i < 5 && counts[i] >= 0; ++i)
                std::cout << counts[i] << " iterations -> steady-state." << std::endl;
    }
    double eta = 0;
    if (shg_efficiency(h, &eta) == SHG_OK) std::cout << "Conversion efficiency = " << std::setprecision(9) << eta << std::endl;
    shg_destroy(h);
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    print_elapsed(el);
    // SHG.cpp:85-97: the elapsed seconds appended to a per-grid timing file
    std::ofstream tf("CPUTime_NZ_" + std::to_string(cfg.nz) + "_N_" + std::to_string(cfg.nx) + "_T.txt",
                     std::ios::app);
    if (tf.is_open()) {
        tf << el << std::endl;
        std::cout << "Data successfully written to the end of the file." << std::endl;
    } else {
        std::cerr << "Unable to open the file for writing." << std::endl;
    }
    return 0;
}
