// Resident z-march variants for 128 x 128 grids.
#include "shg_resident.cuh"

namespace shg {

const float2 *twiddle_symbol_address_resident128() {
    void *p = nullptr;
    cudaGetSymbolAddress(&p, g_twiddle);
    return static_cast<const float2 *>(p);
}
SHG_CHECK_TU(resident128)

SHG_RESIDENT_INSTANTIATE(128, 2, 1, 8)
SHG_RESIDENT_INSTANTIATE(128, 4, 1, 8)
SHG_RESIDENT_INSTANTIATE(128, 4, 2, 8)
SHG_RESIDENT_INSTANTIATE(128, 8, 4, 8)
SHG_RESIDENT_INSTANTIATE(128, 16, 8, 8)

cudaError_t prepare_resident_128(int cs, int minb, int g, int *m) {
    if (g != 8) return cudaErrorInvalidValue;
    if (cs == 2 && minb == 1) return prepare_resident_t<128, 2, 1, 8>(m);
    if (cs == 4 && minb == 1) return prepare_resident_t<128, 4, 1, 8>(m);
    if (cs == 4 && minb == 2) return prepare_resident_t<128, 4, 2, 8>(m);
    if (cs == 8 && minb == 4) return prepare_resident_t<128, 8, 4, 8>(m);
    if (cs == 16 && minb == 8) return prepare_resident_t<128, 16, 8, 8>(m);
    return cudaErrorInvalidValue;
}

cudaError_t launch_resident_128(int cs, int minb, int g, const InstDesc *inst, const int *list, int njobs, int *counter,
                                int max_clusters, cudaStream_t st) {
    if (g != 8) return cudaErrorInvalidValue;
    if (cs == 2 && minb == 1) return launch_resident_t<128, 2, 1, 8>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 4 && minb == 1) return launch_resident_t<128, 4, 1, 8>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 4 && minb == 2) return launch_resident_t<128, 4, 2, 8>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 8 && minb == 4) return launch_resident_t<128, 8, 4, 8>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 16 && minb == 8) return launch_resident_t<128, 16, 8, 8>(inst, list, njobs, counter, max_clusters, st);
    return cudaErrorInvalidValue;
}

}  // namespace shg
