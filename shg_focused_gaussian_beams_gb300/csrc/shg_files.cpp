// Text outputs in the reference's format (Files.h:19-79), written from host copies of the
// device results.
#include <fstream>
#include <iomanip>
#include <string>

#include "shg_internal.h"

namespace shg {

// Files.h:36-57: <name>_r.dat and <name>_i.dat, one line per y, values separated by tabs
// (20 significant digits).
bool save_matrix_complex(const std::string &dir, const std::string &name, const float2 *v, int nx, int ny) {
    for (int part = 0; part < 2; ++part) {
        std::ofstream f(dir + "/" + name + (part == 0 ? "_r.dat" : "_i.dat"));
        if (!f) return false;
        for (int iy = 0; iy < ny; ++iy) {
            for (int ix = 0; ix < nx; ++ix) {
                const float2 c = v[(size_t)iy * nx + ix];
                f << std::setprecision(20) << (part == 0 ? c.x : c.y) << "\t";
            }
            f << "\n";
        }
        if (!f) return false;
    }
    return true;
}

// Files.h:60-79: <name>_<z>.dat per slice, default stream precision.
bool save_tensor_real(const std::string &dir, const std::string &name, const float *T, int nx, int ny, int nz) {
    for (int iz = 0; iz < nz; ++iz) {
        std::ofstream f(dir + "/" + name + "_" + std::to_string(iz) + ".dat");
        if (!f) return false;
        const float *s = T + (size_t)iz * nx * ny;
        for (int iy = 0; iy < ny; ++iy) {
            for (int ix = 0; ix < nx; ++ix) f << s[(size_t)iy * nx + ix] << "\t";
            f << "\n";
        }
        if (!f) return false;
    }
    return true;
}

}  // namespace shg
