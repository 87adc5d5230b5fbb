// Resident z-march variants for 16, 32 and 64 point grids.
#include "shg_resident.cuh"

namespace shg {

const float2 *twiddle_symbol_address_resident() {
    void *p = nullptr;
    cudaGetSymbolAddress(&p, g_twiddle);
    return static_cast<const float2 *>(p);
}
SHG_CHECK_TU(resident64)

SHG_RESIDENT_INSTANTIATE(16, 1, 1, 4)
SHG_RESIDENT_INSTANTIATE(32, 1, 1, 4)
SHG_RESIDENT_INSTANTIATE(64, 1, 1, 8)
SHG_RESIDENT_INSTANTIATE(64, 1, 2, 8)
SHG_RESIDENT_INSTANTIATE(64, 2, 2, 8)
SHG_RESIDENT_INSTANTIATE(64, 2, 4, 8)
SHG_RESIDENT_INSTANTIATE(64, 1, 1, 4)
SHG_RESIDENT_INSTANTIATE(64, 1, 2, 4)
SHG_RESIDENT_INSTANTIATE(64, 4, 4, 8)
SHG_RESIDENT_INSTANTIATE(64, 8, 8, 8)

cudaError_t prepare_resident_small(int n, int cs, int minb, int g, int *m) {
    if (n == 16) return prepare_resident_t<16, 1, 1, 4>(m);
    if (n == 32) return prepare_resident_t<32, 1, 1, 4>(m);
    if (g == 4 && cs == 1 && minb == 1) return prepare_resident_t<64, 1, 1, 4>(m);
    if (g == 4 && cs == 1 && minb == 2) return prepare_resident_t<64, 1, 2, 4>(m);
    if (g != 8) return cudaErrorInvalidValue;
    if (cs == 4 && minb == 4) return prepare_resident_t<64, 4, 4, 8>(m);
    if (cs == 8 && minb == 8) return prepare_resident_t<64, 8, 8, 8>(m);
    if (cs == 1 && minb == 1) return prepare_resident_t<64, 1, 1, 8>(m);
    if (cs == 1 && minb == 2) return prepare_resident_t<64, 1, 2, 8>(m);
    if (cs == 2 && minb == 2) return prepare_resident_t<64, 2, 2, 8>(m);
    if (cs == 2 && minb == 4) return prepare_resident_t<64, 2, 4, 8>(m);
    return cudaErrorInvalidValue;
}

cudaError_t launch_resident_small(int n, int cs, int minb, int g, const InstDesc *inst, const int *list, int njobs,
                                  int *counter, int max_clusters, cudaStream_t st) {
    if (n == 16) return launch_resident_t<16, 1, 1, 4>(inst, list, njobs, counter, max_clusters, st);
    if (n == 32) return launch_resident_t<32, 1, 1, 4>(inst, list, njobs, counter, max_clusters, st);
    if (g == 4 && cs == 1 && minb == 1) return launch_resident_t<64, 1, 1, 4>(inst, list, njobs, counter, max_clusters, st);
    if (g == 4 && cs == 1 && minb == 2) return launch_resident_t<64, 1, 2, 4>(inst, list, njobs, counter, max_clusters, st);
    if (g != 8) return cudaErrorInvalidValue;
    if (cs == 4 && minb == 4) return launch_resident_t<64, 4, 4, 8>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 8 && minb == 8) return launch_resident_t<64, 8, 8, 8>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 1 && minb == 1) return launch_resident_t<64, 1, 1, 8>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 1 && minb == 2) return launch_resident_t<64, 1, 2, 8>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 2 && minb == 2) return launch_resident_t<64, 2, 2, 8>(inst, list, njobs, counter, max_clusters, st);
    if (cs == 2 && minb == 4) return launch_resident_t<64, 2, 4, 8>(inst, list, njobs, counter, max_clusters, st);
    return cudaErrorInvalidValue;
}

}  // namespace shg
