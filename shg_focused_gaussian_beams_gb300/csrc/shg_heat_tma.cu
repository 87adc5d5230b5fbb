// TMA-staged Jacobi sweep (Tfield.h:113-258), bit-identical to the other sweep kernels.
//
// A block owns a 32 (x) x 8 RW (y) tile of columns and a z chunk. One producer thread
// streams the planes of the chunk (and one halo plane on each side) into a four-slot
// shared-memory ring with cp.async.bulk.tensor: per plane a 40 x (8 RW + 2) T box starting
// at (x0 - 4, y0 - 1) (x start rounded down to 16 bytes; out-of-range elements read as zero)
// and the 32 x 8 RW Q/k box of the tile. Eight consumer warps compute RW voxels each per
// plane from the ring (x/y neighbours from plane z, z neighbours from planes z -+ 1) and
// store them. Full and empty mbarriers order the ring; every wait is bounded and a timeout
// sets the caller's error word (one per solve or call, passed to the kernel) that the host
// reads, instead of hanging.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "shg_internal.h"
#include "shg_thermal.cuh"

namespace shg {

namespace {

// Tile: 32 columns x (8 RW) rows, RW rows per consumer warp. T box: 40 x (8 RW + 2) floats
// from (x0 - 4, y0 - 1) (x start rounded down to 16 bytes).
constexpr int TX = 32, BX = 40, XOFF = 4, SLOTS = 4, ZC_DEFAULT = 8;
constexpr int CONSUMER_WARPS = 8;
constexpr int THREADS = 32 * (CONSUMER_WARPS + 1);
template <int RW>
struct TmaTile {
    static constexpr int TY = CONSUMER_WARPS * RW, BY = TY + 2;
    static constexpr int T_BYTES = BX * BY * 4, Q_BYTES = TX * TY * 4;
    static constexpr int T_STRIDE = (T_BYTES + 127) / 128 * 128;  // slots on 128-byte boundaries
    static constexpr int Q_STRIDE = (Q_BYTES + 127) / 128 * 128;
    // ring of T and Q/k slots, full and empty barriers, slack to align the base to 128 bytes
    static constexpr int SMEM = SLOTS * (T_STRIDE + Q_STRIDE) + 2 * SLOTS * 8 + 128;
};
constexpr long long WAIT_LIMIT = 1ll << 18;  // polls before a wait gives up (~3.8 us each: ~1 s)

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false (and *err set to 1) if the phase did not complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, unsigned parity, int *err) {
    for (long long it = 0; it < WAIT_LIMIT; ++it)
        if (mbar_try_wait(b, parity)) return true;
    atomicExch(err, 1);
    return false;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

template <int BC, int RW>
__global__ void __launch_bounds__(THREADS) k_heat_tma(float *__restrict__ Tf, const __grid_constant__ CUtensorMap mT,
                                                     const __grid_constant__ CUtensorMap mQ, const HeatCoef c, int nx,
                                                     int ny, int nz, int zc, int starve, int *err) {
    using G = TmaTile<RW>;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    float *const sT = reinterpret_cast<float *>(base);                          // slot s at s * T_STRIDE
    float *const sQ = reinterpret_cast<float *>(base + SLOTS * G::T_STRIDE);    // slot s at s * Q_STRIDE
    uint64_t *const full = reinterpret_cast<uint64_t *>(base + SLOTS * (G::T_STRIDE + G::Q_STRIDE));
    uint64_t *const empty = full + SLOTS;
    constexpr int TS = G::T_STRIDE / 4, QS = G::Q_STRIDE / 4;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * G::TY;
    const int z0 = blockIdx.z * zc, z1 = min(nz, z0 + zc);
    const int np = (z1 - z0) + 2;  // planes z0-1 .. z1 (relative index i = p - z0 + 1)
    if (threadIdx.x == 0) {
        for (int s = 0; s < SLOTS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], CONSUMER_WARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (warp == CONSUMER_WARPS) {
        // producer: one thread issues the box copies of every plane of the chunk (none when
        // `starve` is set: the failure-detection test of the bounded waits)
        if (lane == 0 && !starve) {
            int issued = 0;
            for (int i = 0; i < np; ++i) {
                const int s = i % SLOTS;
                if (i >= SLOTS && !mbar_wait(&empty[s], ((i / SLOTS) - 1) & 1, err)) break;
                mbar_expect_tx(&full[s], G::T_BYTES + G::Q_BYTES);
                const int p = z0 - 1 + i;
                // the box's x start must be a 16-byte boundary (4 floats): a copy that would
                // start off it is not issued (its waits then run out and report)
                if (!SHG_REQUIRE(((x0 - XOFF) & 3) == 0 && (x0 & 3) == 0, kChkHeatTmaCoord, x0)) break;
                tma_load_3d(sT + s * TS, &mT, x0 - XOFF, y0 - 1, p, &full[s]);
                tma_load_3d(sQ + s * QS, &mQ, x0, y0, p, &full[s]);
                issued = i + 1;
            }
            // copies still in flight complete before the block may exit; only planes that
            // were issued are waited for (after an early break the rest never arrive)
            for (int i = issued - SLOTS < 0 ? 0 : issued - SLOTS; i < issued; ++i)
                mbar_wait(&full[i % SLOTS], (i / SLOTS) & 1, err);
        }
        return;
    }
    // consumers: warp w computes rows y0 + w + 8 r (r < RW) of the tile, lane = column
    const int x = x0 + lane;
    const int sxy = nx * ny;
    bool in[RW], colint[RW];
    int ci[RW];
#pragma unroll
    for (int r = 0; r < RW; ++r) {
        const int ty = warp + CONSUMER_WARPS * r, y = y0 + ty;
        in[r] = x < nx && y < ny;
        colint[r] = x > 0 && x < nx - 1 && y > 0 && y < ny - 1;
        ci[r] = (ty + 1) * BX + lane + XOFF;  // this voxel in a T box
    }
    if (!mbar_wait(&full[0], 0, err) || !mbar_wait(&full[1], 0, err)) return;
    for (int z = z0; z < z1; ++z) {
        const int i = z - z0 + 1;  // relative plane index of z
        const int sm = (i - 1) % SLOTS, s0 = i % SLOTS, sp = (i + 1) % SLOTS;
        if (!mbar_wait(&full[sp], ((i + 1) / SLOTS) & 1, err)) return;
        const float *P = sT + s0 * TS;
        const bool zint = z > 0 && z < nz - 1;
#pragma unroll
        for (int r = 0; r < RW; ++r) {
            const int k = ci[r], y = y0 + warp + CONSUMER_WARPS * r;
            const float zm = sT[sm * TS + k], zp = sT[sp * TS + k];
            const float qk = sQ[s0 * QS + (warp + CONSUMER_WARPS * r) * TX + lane];
            if (in[r]) {
                const int vi = z * sxy + y * nx + x;  // voxel count < 2^31 (checked on the host)
                if (colint[r] && zint) {
                    SHG_AT(Tf, vi, (long long)sxy * nz, kChkHeatVoxel) =
                        interior_voxel(c, P[k - 1], P[k + 1], P[k - BX], P[k + BX], zm, zp, qk);
                } else {
                    float v;
                    if (heat_voxel<BC>(c, x, y, z, nx, ny, nz, P[k - 1], P[k + 1], P[k - BX], P[k + BX], zm, zp, qk,
                                       v))
                        SHG_AT(Tf, vi, (long long)sxy * nz, kChkHeatVoxel) = v;
                }
            }
        }
        // plane i-1 is no longer read by this warp
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[sm]);
    }
}

typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

cudaError_t encoder(EncodeTiled *fn) {
    static EncodeTiled f = nullptr;
    static cudaError_t err = cudaSuccess;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (err == cudaSuccess && q != cudaDriverEntryPointSuccess) err = cudaErrorNotSupported;
        f = reinterpret_cast<EncodeTiled>(p);
    });
    *fn = f;
    return err;
}

// Tensor map of an nx x ny x nz float array (x fastest) with the given box, cached per
// (address, shape, box).
cudaError_t tensor_map(const float *base, int nx, int ny, int nz, int bx, int by, CUtensorMap *out) {
    static std::mutex mu;
    static std::map<std::tuple<const float *, int, int, int, int, int>, CUtensorMap> cache;
    const auto key = std::make_tuple(base, nx, ny, nz, bx, by);
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
        *out = it->second;
        return cudaSuccess;
    }
    EncodeTiled enc = nullptr;
    cudaError_t e = encoder(&enc);
    if (e != cudaSuccess) return e;
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t strides[2] = {(cuuint64_t)nx * 4, (cuuint64_t)nx * ny * 4};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUtensorMap m;
    const CUresult r = enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    cache[key] = m;
    *out = m;
    return cudaSuccess;
}

}  // namespace

SHG_CHECK_TU(heat_tma)

// Planes per block: a block streams its chunk plus one halo plane on each side. At
// 256x256x400 on GB300 with 4 rows per warp, chunks of 4, 6, 8, 16, 32 planes take 71.2,
// 69.9, 70.0, 72.5, 80.1 us per sweep (short chunks: more blocks, more copies in flight;
// shorter still: more halo planes). SHG_HEAT_ZC overrides the default of 8.
int heat_tma_chunk(int nz) {
    int v = ZC_DEFAULT;
    if (const char *e = std::getenv("SHG_HEAT_ZC")) v = std::max(1, std::atoi(e));
    return std::min(v, nz);
}

template <int RW>
cudaError_t launch_heat_tma_t(float *Tf, const float *Ti, const float *QK, const HeatCoef &c, int nx, int ny,
                              int nz, int bc, int *err, cudaStream_t st) {
    using G = TmaTile<RW>;
    CUtensorMap mT, mQ;
    cudaError_t e = tensor_map(Ti, nx, ny, nz, BX, G::BY, &mT);
    if (e != cudaSuccess) return e;
    e = tensor_map(QK, nx, ny, nz, TX, G::TY, &mQ);
    if (e != cudaSuccess) return e;
    const int zc = heat_tma_chunk(nz);
    const dim3 grid((nx + TX - 1) / TX, (ny + G::TY - 1) / G::TY, (nz + zc - 1) / zc);
    auto *k = bc == 0 ? k_heat_tma<0, RW> : k_heat_tma<1, RW>;
    if (G::SMEM > 48 * 1024) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM);
        if (e != cudaSuccess) return e;
    }
    // SHG_HEAT_TMA_STARVE=1: the producer issues no copies, so every consumer wait runs out
    // and sets the error flag (tests the bounded waits and the host's check; no sweep result)
    const char *sv = std::getenv("SHG_HEAT_TMA_STARVE");
    const int starve = sv && std::atoi(sv) == 1 ? 1 : 0;
    k<<<grid, THREADS, G::SMEM, st>>>(Tf, mT, mQ, c, nx, ny, nz, zc, starve, err);
    return cudaGetLastError();
}

bool heat_tma_supported(int nx, int ny, int nz) {
    // 16-byte row and plane strides, 16-byte aligned bases (cudaMalloc), 32-bit offsets
    return nx % 4 == 0 && nx >= 8 && ny >= 2 && nz >= 2 && (long long)nx * ny * nz < (1ll << 31);
}

cudaError_t launch_heat_tma(float *Tf, const float *Ti, const float *QK, const HeatCoef &c, int nx, int ny, int nz,
                            int bc, int *err, cudaStream_t st, int rows_per_warp) {
    if (!heat_tma_supported(nx, ny, nz) || !err || (reinterpret_cast<uintptr_t>(Ti) & 15) ||
        (reinterpret_cast<uintptr_t>(QK) & 15))
        return cudaErrorInvalidValue;
    switch (rows_per_warp) {
        case 1: return launch_heat_tma_t<1>(Tf, Ti, QK, c, nx, ny, nz, bc, err, st);
        case 2: return launch_heat_tma_t<2>(Tf, Ti, QK, c, nx, ny, nz, bc, err, st);
        case 4: return launch_heat_tma_t<4>(Tf, Ti, QK, c, nx, ny, nz, bc, err, st);
        case 8: return launch_heat_tma_t<8>(Tf, Ti, QK, c, nx, ny, nz, bc, err, st);
        default: return cudaErrorInvalidValue;
    }
}

// Reads and clears the error word `err` on `st` (1: a wait gave up, the sweep is incomplete).
cudaError_t heat_tma_error(int *err, int *flag, cudaStream_t st) {
    cudaError_t e = cudaMemcpyAsync(flag, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

// Error words of component calls that own no solve (shg_heat_sweeps_device): a pool of
// device ints, each leased to one call at a time and returned cleared.
namespace {
std::mutex g_err_mu;
std::map<int, std::vector<int *>> g_err_free;  // per device ordinal
}  // namespace

cudaError_t heat_error_word_acquire(int **err) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    {
        std::lock_guard<std::mutex> lock(g_err_mu);
        auto &v = g_err_free[dev];
        if (!v.empty()) {
            *err = v.back();
            v.pop_back();
            return cudaSuccess;
        }
    }
    int *p = nullptr;
    e = cudaMalloc(&p, sizeof(int));
    if (e != cudaSuccess) return e;
    e = cudaMemset(p, 0, sizeof(int));
    if (e != cudaSuccess) {
        cudaFree(p);
        return e;
    }
    *err = p;
    return cudaSuccess;
}

void heat_error_word_release(int *err) {
    int dev = 0;
    if (!err || cudaGetDevice(&dev) != cudaSuccess) return;
    std::lock_guard<std::mutex> lock(g_err_mu);
    g_err_free[dev].push_back(err);
}

}  // namespace shg
