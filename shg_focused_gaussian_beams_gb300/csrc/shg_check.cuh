// Device-side checks of the SHG_CHECK build (build.py, variant "check"; normal builds
// compile every check away).
//
// A check never traps and never lets a bad access through: a failed SHG_REQUIRE records
// (site, value) in the translation unit's status word (first failure wins) and returns
// false so the caller can skip the work; SHG_AT redirects an out-of-range access to a
// scratch sink. The host reads and clears the words with shg_check_status (include/shg.h)
// after synchronising the device. Sites name the kernel and the index kind, so a report
// says where the arithmetic went wrong without a device fault.
#pragma once

#include <cuda_runtime.h>

namespace shg {

enum CheckSite : int {
    kChkSelfTest = 1,
    kChkDescriptor = 2,    // descriptor grid size differs from the kernel's template N
    kChkStage = 3,         // SSFM stage outside [0, nsteps] or nsteps >= nz
    kChkList = 4,          // solve list entry or job index out of range
    kChkClusterRank = 5,   // distributed-shared-memory rank outside the cluster
    kChkRowsGlobal = 10,   // streaming row pass, field index
    kChkColsGlobal = 11,   // streaming column pass, field index
    kChkPropagator = 12,   // propagator index
    kChkSlices = 13,       // per-slice capture index
    kChkResidentRow = 20,  // resident march, local row index
    kChkResidentCol = 21,  // resident march, remote column element
    kChkResidentLoad = 22, // resident march, field load / output index
    kChkClusterPtRow = 30, // cluster march, local row index
    kChkClusterPtCol = 31, // cluster march, remote column element
    kChkCoop = 40,         // persistent grid, row unit / column group
    kChkHeatVoxel = 50,    // heat sweep, voxel index
    kChkHeatTmaCoord = 51, // TMA heat sweep, box coordinate (alignment or range)
    kChkThermalRows = 60,  // THERMAL row pass, field or temperature index
    kChkAdjoint = 70,      // adjoint kernels, field or checkpoint index
};

#ifdef SHG_CHECK
constexpr bool kCheckBuild = true;
static __device__ unsigned long long g_check_word;
static __device__ float4 g_check_sink[4];

// First failure of this translation unit: site in bits 48..63, value in bits 0..47.
static __device__ __noinline__ void check_fail(int site, long long value) {
    const unsigned long long w =
        ((unsigned long long)(unsigned)(site & 0xffff) << 48) | ((unsigned long long)value & 0xffffffffffffull);
    atomicCAS(&g_check_word, 0ull, w);
}

template <class T>
__device__ __forceinline__ T *check_ptr(T *p, long long i, long long n, int site) {
    if (i >= 0 && i < n) return p + i;
    check_fail(site, i);
    return reinterpret_cast<T *>(g_check_sink);
}

#define SHG_REQUIRE(cond, site, value) ((cond) ? true : (::shg::check_fail((site), (long long)(value)), false))
#define SHG_AT(p, i, n, site) (*::shg::check_ptr((p), (long long)(i), (long long)(n), (site)))
// Host accessor of this translation unit's word (read and cleared; device synchronised by
// the caller).
#define SHG_CHECK_TU(name)                                                          \
    unsigned long long check_word_take_##name() {                                  \
        unsigned long long w = 0, z = 0;                                            \
        if (cudaMemcpyFromSymbol(&w, g_check_word, sizeof(w)) != cudaSuccess) return ~0ull; \
        cudaMemcpyToSymbol(g_check_word, &z, sizeof(z));                            \
        return w;                                                                   \
    }
#else
constexpr bool kCheckBuild = false;
#define SHG_REQUIRE(cond, site, value) true
#define SHG_AT(p, i, n, site) ((p)[i])
#define SHG_CHECK_TU(name) \
    unsigned long long check_word_take_##name() { return 0; }
#endif

}  // namespace shg
