// Resident z-march variants for 256 x 256 grids.
#include "shg_resident.cuh"

namespace shg {

const float2 *twiddle_symbol_address_resident256() {
    void *p = nullptr;
    cudaGetSymbolAddress(&p, g_twiddle);
    return static_cast<const float2 *>(p);
}
SHG_CHECK_TU(resident256)

SHG_RESIDENT_INSTANTIATE(256, 8, 1, 16)
SHG_RESIDENT_INSTANTIATE(256, 16, 1, 16)
SHG_RESIDENT_INSTANTIATE(256, 16, 2, 16)

cudaError_t prepare_resident_256(int cs, int minb, int g, int *m) {
    if (g != 16) return cudaErrorInvalidValue;
    if (cs == 8 && minb == 1) return prepare_resident_t<256, 8, 1, 16>(m);
    if (cs == 16 && minb == 1) return prepare_resident_t<256, 16, 1, 16>(m);
    if (cs == 16 && minb == 2) return prepare_resident_t<256, 16, 2, 16>(m);
    return cudaErrorInvalidValue;
}

cudaError_t launch_resident_256(int cs, int minb, int g, const InstDesc *inst, const int *list, int njobs, int *counter,
                                int max_clusters, cudaStream_t st) {
    if (g != 16) return cudaErrorInvalidValue;
    if (cs == 8 && minb == 1) return launch_resident_t<256, 8, 1, 16>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 16 && minb == 1) return launch_resident_t<256, 16, 1, 16>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 16 && minb == 2) return launch_resident_t<256, 16, 2, 16>(inst, list, njobs, counter, max_clusters, st);
    return cudaErrorInvalidValue;
}

}  // namespace shg
