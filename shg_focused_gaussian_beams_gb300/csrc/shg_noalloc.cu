// Plain CWES without any device allocation.
//
// Some callers cannot call cudaMalloc: hosts whose device memory is owned up front by
// another allocator (a framework that reserves the whole pool at start-up), latency-bound
// control loops that must not stall or fail on an allocation mid-run, and plugin hosts
// that forbid device allocation from extension code. shg_cwes_noalloc serves them: the
// caller passes device buffers for the input and output fields, and all working memory
// of the march (working fields, shifted propagators, per-slice constants, the solve
// descriptor and the power sums) lives in one file-scope device array of fixed size.
//
// Limits: NX = NY a power of two in [16, 128], NZ in [2, 4096]. The array (see
// kNoAllocBytes) is part of the library's device image, so every GPU that loads the
// library holds it until the process exits.
//
// Sharing: every call uses the same array, and it keeps the last call's contents; the
// parts that must start at zero (power sums, the SH field when no SH input is given) are
// cleared by each call. Calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array and must be serialised by the caller.
//
// Set-up: the first call on a device, with that device current, looks up the array's
// device address (cudaGetSymbolAddress) and uploads the FFT twiddle tables with a
// blocking copy; make that first call before any stream capture. Both are cached per
// device ordinal for the life of the process, so a device reset (cudaDeviceReset, or a
// new primary context) after the first call is not supported.
//
// The call's own parameters (the solve descriptor) reach the device as a kernel argument
// of a one-thread staging kernel, so no copy reads host memory after the call returns.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "shg_internal.h"
#include "shg_march.cuh"

namespace shg {
namespace {

constexpr int kNoAllocMaxN = 128;
constexpr int kNoAllocMaxNz = 4096;
constexpr size_t kFieldBytes = (size_t)kNoAllocMaxN * kNoAllocMaxN * sizeof(float2);  // 128 KiB
constexpr size_t kStepBytes = (size_t)kNoAllocMaxNz * sizeof(float4);                // 64 KiB
constexpr size_t kOffP = 0, kOffS = kFieldBytes, kOffHp = 2 * kFieldBytes, kOffHs = 3 * kFieldBytes;
constexpr size_t kOffStep = 4 * kFieldBytes;
constexpr size_t kOffAcc = kOffStep + kStepBytes;      // 4 doubles
constexpr size_t kOffDesc = kOffAcc + 256;             // one InstDesc
constexpr size_t kOffList = kOffDesc + 1024;           // one int
constexpr size_t kNoAllocBytes = kOffList + 256;       // 576 KiB + 1.5 KiB
static_assert(sizeof(InstDesc) <= 1024, "descriptor slot too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `dev` (current), looked up once per device.
int scratch_for(int dev, unsigned char **out) {
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("shg_cwes_noalloc: device ordinal out of range");
        return SHG_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error(std::string("shg_cwes_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return SHG_ERR_CUDA;
        }
        g_scratch_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_addr[dev];
    return SHG_OK;
}

// Writes the solve descriptor and the one-entry solve list into the scratch array and
// clears the power sums. The descriptor travels by value as a kernel argument.
__global__ void k_noalloc_stage(InstDesc d, InstDesc *dst, int *list) {
    if (threadIdx.x == 0) {
        *dst = d;
        list[0] = 0;
        d.acc[0] = d.acc[1] = d.acc[2] = d.acc[3] = 0.0;
    }
}

}  // namespace
}  // namespace shg

using namespace shg;

#define NOALLOC_CUDA(call)                                                                        \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            set_error(std::string("shg_cwes_noalloc: ") + #call + ": " + cudaGetErrorString(e_)); \
            return SHG_ERR_CUDA;                                                                  \
        }                                                                                         \
    } while (0)

extern "C" int shg_cwes_noalloc(const shg_config *cfg, float temp, const void *pump_in, const void *sh_in,
                                void *pump_out, void *sh_out, double *eta, void *stream) {
    if (!cfg || !pump_in || !pump_out || !sh_out) {
        set_error("shg_cwes_noalloc: null argument");
        return SHG_ERR_INVALID;
    }
    const int n = cfg->nx;
    if (cfg->nx != cfg->ny || n < 16 || n > kNoAllocMaxN || (n & (n - 1)) != 0) {
        set_error("shg_cwes_noalloc: grid must be square with NX = NY a power of two in [16, " +
                  std::to_string(kNoAllocMaxN) + "] (fixed scratch size)");
        return SHG_ERR_INVALID;
    }
    if (cfg->nz < 2 || cfg->nz > kNoAllocMaxNz) {
        set_error("shg_cwes_noalloc: NZ must be in [2, " + std::to_string(kNoAllocMaxNz) + "] (fixed scratch size)");
        return SHG_ERR_INVALID;
    }
    if (cfg->crystal != SHG_CRYSTAL_SPPLT && cfg->crystal != SHG_CRYSTAL_PPLN) {
        set_error("shg_cwes_noalloc: unknown crystal");
        return SHG_ERR_INVALID;
    }
    if (!(cfg->lx > 0) || !(cfg->ly > 0) || !(cfg->lz > 0)) {
        set_error("shg_cwes_noalloc: window and crystal length must be positive");
        return SHG_ERR_INVALID;
    }
    int dev = 0;
    NOALLOC_CUDA(cudaGetDevice(&dev));
    unsigned char *base = nullptr;
    int rc = scratch_for(dev, &base);
    if (rc) return rc;
    rc = ensure_twiddles(dev);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    InstDesc d;
    std::memset(&d, 0, sizeof(d));
    SolveParams sp{n, cfg->nz, cfg->lx, cfg->ly, 1.0f, 1.0f, 0.5f * cfg->lz, temp, temp, temp};
    fill_scalars(*cfg, sp, d);
    d.P = reinterpret_cast<float2 *>(base + kOffP);
    d.S = reinterpret_cast<float2 *>(base + kOffS);
    d.Hp = reinterpret_cast<float2 *>(base + kOffHp);
    d.Hs = reinterpret_cast<float2 *>(base + kOffHs);
    d.stepc = reinterpret_cast<float4 *>(base + kOffStep);
    d.acc = reinterpret_cast<double *>(base + kOffAcc);
    d.Pout = static_cast<float2 *>(pump_out);
    d.Sout = static_cast<float2 *>(sh_out);
    d.pump_given = 1;
    InstDesc *d_desc = reinterpret_cast<InstDesc *>(base + kOffDesc);
    int *d_list = reinterpret_cast<int *>(base + kOffList);
    const size_t bytes = (size_t)n * n * sizeof(float2);

    k_noalloc_stage<<<1, 32, 0, st>>>(d, d_desc, d_list);
    NOALLOC_CUDA(cudaGetLastError());
    NOALLOC_CUDA(cudaMemcpyAsync(d.P, pump_in, bytes, cudaMemcpyDeviceToDevice, st));
    if (sh_in)
        NOALLOC_CUDA(cudaMemcpyAsync(d.S, sh_in, bytes, cudaMemcpyDeviceToDevice, st));
    else
        NOALLOC_CUDA(cudaMemsetAsync(d.S, 0, bytes, st));
    NOALLOC_CUDA(launch_setup(d_desc, 1, n * n, cfg->nz, st));
    const int K = cfg->nz - 1;
    for (int s = 0; s <= K; ++s) {
        NOALLOC_CUDA(launch_rows(n, d_desc, d_list, 1, s, st));
        if (s < K) NOALLOC_CUDA(launch_cols(n, d_desc, d_list, 1, st));
    }
    if (eta) {
        double acc[4] = {0, 0, 0, 0};
        NOALLOC_CUDA(cudaMemcpyAsync(acc, d.acc, sizeof(acc), cudaMemcpyDeviceToHost, st));
        NOALLOC_CUDA(cudaStreamSynchronize(st));
        const float np_t = crystal_index(cfg->crystal, cfg->lp, temp),
                    ns_t = crystal_index(cfg->crystal, (float)(0.5 * (double)cfg->lp), temp);
        *eta = field_power(acc[1], ns_t, d.dx, d.dy) / field_power(acc[0], np_t, d.dx, d.dy);
    }
    return SHG_OK;
}
