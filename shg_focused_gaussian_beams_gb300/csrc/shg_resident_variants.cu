// Resident z-march: every solve keeps both fields in shared memory for its whole march.
//
// A solve of N x N points is owned by a thread-block cluster of CS CTAs (variants: CS = 1,
// 2, 4 or 8 for N = 64, 2, 4, 8 or 16 for N = 128, 8 or 16 for N = 256; the large clusters
// spread one solve over more SMs, which shortens a lone solve); CTA r of the cluster holds rows
// [r*R, (r+1)*R), R = N / CS, of the pump and SH fields. Per SSFM step:
//   row phase (local):   forward FFT along x finishing step s-1, RK4(z_{s-1}),
//                        [capture at the top of slice nz-1], RK4(z_s), backward FFT;
//   cluster barrier;
//   column phase:        CTA r transforms columns [r*R, (r+1)*R): each column is read
//                        from the CTAs that own its rows (distributed shared memory),
//                        backward FFT along y, shifted propagator, forward FFT, and
//                        written back in place;
//   cluster barrier.
// The arithmetic (line FFTs, RK4, propagator product) is the same device code as the
// streaming row/column kernels of shg_march.cu, so results are bit-identical; only the
// storage moves from global memory to shared memory, removing the per-step global
// traffic and the two launches per step.
//
// The kernel is persistent: each cluster takes solves of its size class from a queue
// (an atomic counter over the class list, ordered by work, largest first) until none is
// left. No cluster waits on another, so a cluster that starts late only finds fewer solves.
//
// The kernel template lives in shg_resident.cuh and is instantiated per grid size in
// shg_resident_{64,128,256}.cu; this file lists the variants (cluster size CS, CTAs per SM
// MINB, and the line-FFT split G: E = N/G point register DFTs, then G-point ones) that the
// batch schedule's autotuner times, and dispatches to them.
#include <cuda_runtime.h>

#include "shg_internal.h"

namespace shg {

cudaError_t prepare_resident_small(int n, int cs, int minb, int g, int *max_clusters);
cudaError_t launch_resident_small(int n, int cs, int minb, int g, const InstDesc *inst, const int *list, int njobs,
                                  int *counter, int max_clusters, cudaStream_t st);
cudaError_t prepare_resident_128(int cs, int minb, int g, int *max_clusters);
cudaError_t launch_resident_128(int cs, int minb, int g, const InstDesc *inst, const int *list, int njobs, int *counter,
                                int max_clusters, cudaStream_t st);
cudaError_t prepare_resident_256(int cs, int minb, int g, int *max_clusters);
cudaError_t launch_resident_256(int cs, int minb, int g, const InstDesc *inst, const int *list, int njobs, int *counter,
                                int max_clusters, cudaStream_t st);

int resident_variants(int n, ResidentVariant *out, int max_out) {
    static const ResidentVariant v16[] = {{1, 1, 4}};
    static const ResidentVariant v64[] = {{1, 1, 8}, {1, 2, 8}, {2, 2, 8}, {2, 4, 8}, {1, 1, 4}, {1, 2, 4},
                                          {4, 4, 8}, {8, 8, 8}};
    static const ResidentVariant v128[] = {{2, 1, 8}, {4, 1, 8}, {4, 2, 8}, {8, 4, 8}, {16, 8, 8}};
    static const ResidentVariant v256[] = {{8, 1, 16}, {16, 1, 16}, {16, 2, 16}};
    const ResidentVariant *v = nullptr;
    int c = 0;
    switch (n) {
        case 16: case 32: v = v16; c = 1; break;
        case 64: v = v64; c = 8; break;
        case 128: v = v128; c = 5; break;
        case 256: v = v256; c = 3; break;
        default: return 0;
    }
    for (int i = 0; i < c && i < max_out; ++i) out[i] = v[i];
    return c < max_out ? c : max_out;
}

ResidentVariant resident_default(int n) {
    ResidentVariant v{1, 1, 0};
    resident_variants(n, &v, 1);
    return v;
}

cudaError_t prepare_resident(int n, ResidentVariant v, int *max_clusters) {
    if (v.cs == 0) {  // the persistent cooperative grid of one solve: does it fit co-resident?
        const cudaError_t e = launch_coop(n, nullptr, nullptr, nullptr, nullptr, nullptr);
        *max_clusters = e == cudaSuccess ? 1 : 0;
        return e;
    }
    if (v.cs == -1) return prepare_cluster_pt(n, max_clusters);
    switch (n) {
        case 16: case 32: case 64: return prepare_resident_small(n, v.cs, v.minb, v.g, max_clusters);
        case 128: return prepare_resident_128(v.cs, v.minb, v.g, max_clusters);
        case 256: return prepare_resident_256(v.cs, v.minb, v.g, max_clusters);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_resident(int n, ResidentVariant v, const InstDesc *inst, const int *list, int njobs, int *counter,
                            int max_clusters, cudaStream_t st) {
    if (v.cs == -1) return launch_cluster_pt(n, inst, list, njobs, st);  // one cluster per solve
    switch (n) {
        case 16: case 32: case 64:
            return launch_resident_small(n, v.cs, v.minb, v.g, inst, list, njobs, counter, max_clusters, st);
        case 128: return launch_resident_128(v.cs, v.minb, v.g, inst, list, njobs, counter, max_clusters, st);
        case 256: return launch_resident_256(v.cs, v.minb, v.g, inst, list, njobs, counter, max_clusters, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace shg
