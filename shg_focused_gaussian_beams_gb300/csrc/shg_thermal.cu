// THERMAL kernels (-DTHERMAL of the reference): temperature set-up, the steady heat
// Jacobi sweep, its convergence sum, the Sellmeier / delta-k(T) tables, and the thermal
// row pass of the z-march (per-pixel coupling from T, running delta-k sum, heat source).
//
// The heat sweep reproduces Tfield.h:113-258 bit for bit: the same float operations in
// the same order with no contraction (__fadd_rn / __fmul_rn / __fdiv_rn), and the double
// sub-expressions of the edge formulas in double. The Sellmeier index is evaluated in
// double exactly as Crystal.h:116-132 does on the host (the reference's own arithmetic),
// so delta-k(T) is bit-identical too.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdlib>
#include <string>

#include "shg_internal.h"
#include "shg_coop.cuh"
#include "shg_thermal.cuh"

namespace shg {

const float2 *twiddle_symbol_address_thermal() {
    void *p = nullptr;
    cudaGetSymbolAddress(&p, g_twiddle);
    return static_cast<const float2 *>(p);
}
SHG_CHECK_TU(thermal)

// ---------------------------------------------------------------------------------------
// Tfield.h:31-110: T = Temp everywhere, then the oven faces (bc 0: y = 0 plane; bc 1: all
// four lateral faces), T1 for z < NZ/2 and T2 otherwise.
__global__ void k_init_temperature(float *T, int nx, int ny, int nz, float temp, float t1, float t2, int bc) {
    const size_t total = (size_t)nx * ny * nz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((size_t)nx * ny));
        const bool oven = bc == 0 ? (y == 0) : (y == 0 || y == ny - 1 || x == 0 || x == nx - 1);
        const double half = (double)(float)nz / 2.0;
        T[i] = oven ? ((double)z < half ? t1 : t2) : temp;
    }
}

// One Jacobi sweep Tf <- stencil(Ti). Voxels the reference never writes are left alone;
// both ping-pong buffers start equal, so they hold the same value.
template <int BC>
__global__ void __launch_bounds__(256) k_heat(float *__restrict__ Tf, const float *__restrict__ Ti,
                                              const float *__restrict__ QK, const HeatCoef c, int nx, int ny, int nz) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= nx || y >= ny) return;
    const size_t sxy = (size_t)nx * ny;
    const size_t i = (size_t)z * sxy + (size_t)y * nx + x;
    const bool xi = x > 0 && x < nx - 1, yi = y > 0 && y < ny - 1, zi = z > 0 && z < nz - 1;
    const float *t = Ti + i;
    const long long X = 1, Y = nx, Z = (long long)sxy;
    if (xi && yi && zi) {
        const float a = __fdiv_rn(__fadd_rn(t[X], t[-X]), c.dx2);
        const float b = __fdiv_rn(__fadd_rn(t[Y], t[-Y]), c.dy2);
        const float d = __fdiv_rn(__fadd_rn(t[Z], t[-Z]), c.dz2);
        Tf[i] = __fmul_rn(c.L2, __fadd_rn(__fadd_rn(__fadd_rn(a, b), d), QK[i]));
        return;
    }
    if (xi && yi) {  // z = 0 or z = NZ-1 (back / front faces)
        const long long zn = z == 0 ? Z : -Z;
        float s = __fadd_rn(t[zn], __fmul_rn(c.az, __fadd_rn(t[X], t[-X])));
        s = __fadd_rn(s, __fmul_rn(c.bz, __fadd_rn(t[Y], t[-Y])));
        s = __fadd_rn(s, c.tinfBiz);
        Tf[i] = __fdiv_rn(s, c.den_z);
        return;
    }
    if (BC != 0) return;  // oven surrounded: lateral faces are fixed
    const bool xe = x == 0 || x == nx - 1, ze = z == 0 || z == nz - 1, ytop = y == ny - 1;
    const long long xn = x == 0 ? X : -X;
    const long long zn = z == 0 ? Z : -Z;
    if (xe && yi && zi) {  // left / right faces
        float s = __fadd_rn(t[xn], __fmul_rn(c.ax, __fadd_rn(t[Y], t[-Y])));
        s = __fadd_rn(s, __fmul_rn(c.bx, __fadd_rn(t[Z], t[-Z])));
        s = __fadd_rn(s, c.tinfBix);
        Tf[i] = __fdiv_rn(s, c.den_x);
    } else if (xi && ytop && zi) {  // top face
        float s = __fadd_rn(t[-Y], __fmul_rn(c.ay, __fadd_rn(t[X], t[-X])));
        s = __fadd_rn(s, __fmul_rn(c.by, __fadd_rn(t[Z], t[-Z])));
        s = __fadd_rn(s, c.tinfBiy);
        Tf[i] = __fdiv_rn(s, c.den_y);
    } else if (xe && yi && ze) {  // vertical sides
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(c.av, t[xn]), __fmul_rn(c.bv, t[zn])),
                                  __fmul_rn(c.cv, __fadd_rn(t[Y], t[-Y])));
        Tf[i] = __double2float_rn(__dmul_rn(__dadd_rn((double)s, c.KV), (double)c.V));
    } else if (ytop && xi && ze) {  // horizontal sides
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(c.ah, t[-Y]), __fmul_rn(c.bh, t[zn])),
                                  __fmul_rn(c.ch, __fadd_rn(t[-X], t[X])));
        Tf[i] = __double2float_rn(__dmul_rn(__dadd_rn((double)s, c.KH), (double)c.H));
    } else if (xe && ytop && zi) {  // depth sides
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(c.ad, t[-Y]), __fmul_rn(c.bd, t[xn])),
                                  __fmul_rn(c.cd, __fadd_rn(t[Z], t[-Z])));
        Tf[i] = __double2float_rn(__dmul_rn(__dadd_rn((double)s, c.KD), (double)c.D));
    } else if (xe && ytop && ze) {  // vertices
        float s = __fadd_rn(__fmul_rn(c.AV, t[xn]), __fmul_rn(c.BV, t[-Y]));
        s = __fadd_rn(s, __fmul_rn(c.CV, t[zn]));
        s = __fadd_rn(s, c.tinfBiD);
        Tf[i] = __fmul_rn(s, c.GV);
    }
}

// Exhaustive check of the corrected product against IEEE division for every float of
// either sign with biased exponent in [kDivExpLo, kDivExpHi]: counts mismatches.
__global__ void k_verify_div(float d, float r, unsigned long long *mismatch) {
    const unsigned long long span = (unsigned long long)(kDivExpHi - kDivExpLo + 1) << 23;
    unsigned long long bad = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < 2 * span;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned sign = i >= span ? 0x80000000u : 0u;
        const unsigned bits = sign | (unsigned)(((unsigned long long)kDivExpLo << 23) + (i % span));
        const float a = __uint_as_float(bits);
        const float q1 = __fdiv_rn(a, d);
        const float q = a * r;
        const float rem = fmaf(-q, d, a);
        const float q2 = fmaf(rem, r, q);
        bad += __float_as_uint(q1) != __float_as_uint(q2);
    }
    for (int o = 16; o > 0; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(mismatch, bad);
}

cudaError_t verify_fast_division(float d, float r, unsigned long long *d_count, unsigned long long *mismatches,
                                 cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    k_verify_div<<<1216, 256, 0, st>>>(d, r, d_count);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(mismatches, d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

// 2.5D form of the same sweep: a 32x8 (x, y) tile marches a z range; each thread keeps
// T(z-1), T(z), T(z+1) of its column in registers and reads its x / y neighbours from a
// shared-memory copy of the current plane with a one-voxel halo. Every global load (the
// column's T, Q/k and the halo values) is issued two planes before it is used, so the
// DRAM latency overlaps the work of the planes in between instead of sitting between the
// two barriers of one plane.
constexpr int HT_X = 32, HT_Y = 8, HT_Z = 25;
template <int BC>
__global__ void __launch_bounds__(HT_X * HT_Y) k_heat25(float *__restrict__ Tf, const float *__restrict__ Ti,
                                                        const float *__restrict__ QK, const HeatCoef c, int nx, int ny,
                                                        int nz) {
    __shared__ float pl[HT_Y + 2][HT_X + 2];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = blockIdx.x * HT_X + tx, y = blockIdx.y * HT_Y + ty;
    const int z0 = blockIdx.z * HT_Z, z1 = min(nz, z0 + HT_Z);
    const bool in = x < nx && y < ny;
    const size_t sxy = (size_t)nx * ny;
    const size_t col = (size_t)y * nx + x;
    // halo roles: a neighbour row (y-1 or y+1) and a neighbour column (x-1 or x+1)
    int hx = -1, hy = -1, sx = 0, sy = 0;
    if (ty == 0 && y > 0) { hx = x; hy = y - 1; sx = tx + 1; sy = 0; }
    if (ty == HT_Y - 1 && y + 1 < ny) { hx = x; hy = y + 1; sx = tx + 1; sy = HT_Y + 1; }
    int hx2 = -1, hy2 = -1, sx2 = 0, sy2 = 0;
    if (tx == 0 && x > 0) { hx2 = x - 1; hy2 = y; sx2 = 0; sy2 = ty + 1; }
    if (tx == HT_X - 1 && x + 1 < nx) { hx2 = x + 1; hy2 = y; sx2 = HT_X + 1; sy2 = ty + 1; }
    const bool h1 = in && hx >= 0, h2 = in && hx2 >= 0;
    const size_t hcol = h1 ? (size_t)hy * nx + hx : 0, hcol2 = h2 ? (size_t)hy2 * nx + hx2 : 0;
    // column pointers advance by one plane per step
    const float *pT = Ti + col, *pH = Ti + hcol, *pH2 = Ti + hcol2, *pQ = QK + col;
    float *pO = Tf + col;
    auto ldT = [&](int z) { return (in && z >= 0 && z < nz) ? pT[(size_t)z * sxy] : 0.f; };
    float tm = ldT(z0 - 1), tc = ldT(z0), tp = ldT(z0 + 1), f1 = ldT(z0 + 2);
    const float *qz = pQ + (size_t)z0 * sxy, *tz3 = pT + (size_t)(z0 + 3) * sxy;
    const float *hz = pH + (size_t)z0 * sxy, *hz2 = pH2 + (size_t)z0 * sxy;
    float *oz = pO + (size_t)z0 * sxy;
    float q0 = (in && z0 < z1) ? qz[0] : 0.f, q1 = (in && z0 + 1 < z1) ? qz[sxy] : 0.f;
    float a0 = (h1 && z0 < z1) ? hz[0] : 0.f, a1 = (h1 && z0 + 1 < z1) ? hz[sxy] : 0.f;
    float b0 = (h2 && z0 < z1) ? hz2[0] : 0.f, b1 = (h2 && z0 + 1 < z1) ? hz2[sxy] : 0.f;
    const size_t two = 2 * sxy;
    for (int z = z0; z < z1; ++z) {
        const float f2 = (in && z + 3 < nz) ? *tz3 : 0.f;
        const bool nx2 = z + 2 < z1;
        const float q2 = (in && nx2) ? qz[two] : 0.f;
        const float a2 = (h1 && nx2) ? hz[two] : 0.f;
        const float b2 = (h2 && nx2) ? hz2[two] : 0.f;
        tz3 += sxy;
        qz += sxy;
        hz += sxy;
        hz2 += sxy;
        pl[ty + 1][tx + 1] = tc;
        if (h1) pl[sy][sx] = a0;
        if (h2) pl[sy2][sx2] = b0;
        __syncthreads();
        if (in) {
            float out;
            if (heat_voxel<BC>(c, x, y, z, nx, ny, nz, pl[ty + 1][tx], pl[ty + 1][tx + 2], pl[ty][tx + 1],
                               pl[ty + 2][tx + 1], tm, tp, q0, out))
                *oz = out;
        }
        oz += sxy;
        __syncthreads();
        tm = tc;
        tc = tp;
        tp = f1;
        f1 = f2;
        q0 = q1;
        q1 = q2;
        a0 = a1;
        a1 = a2;
        b0 = b1;
        b1 = b2;
    }
}

// Warp-strip form of the same sweep: a warp owns a 32 (x) x RY (y) strip of columns and
// marches a z range with no block-level synchronisation. Each lane keeps its column's RY
// values of planes z-1, z, z+1 in registers (y neighbours inside the strip come from
// registers, x neighbours from the adjacent lanes by shuffle); the two y-halo rows and the
// 2 RY x-halo values (spread over lanes 0..RY-1 and 16..16+RY-1, then shuffled to lanes 0
// and 31) are loaded per plane. All loads of plane z+1 (z+2 for the column values) are
// issued before plane z is computed. Strips away from the x and y faces take the interior
// formula for z-interior planes; other voxels go through heat_voxel.
constexpr int WS_WARPS = 4;


template <int BC, int RY, int MINB>
__global__ void __launch_bounds__(32 * WS_WARPS, MINB) k_heat_ws(float *__restrict__ Tf, const float *__restrict__ Ti,
                                                          const float *__restrict__ QK, const HeatCoef c, int nx,
                                                          int ny, int nz, int zc) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 32, x = x0 + lane;
    const int y0 = (blockIdx.y * WS_WARPS + w) * RY;
    if (y0 >= ny) return;  // uniform per warp; no block barrier below
    const int z0 = blockIdx.z * zc, z1 = min(nz, z0 + zc);
    const int sxy = nx * ny;
    const bool xin = x < nx;
    const bool wint = x0 >= 1 && x0 + 31 <= nx - 2 && y0 >= 1 && y0 + RY - 1 <= ny - 2;
    // per-lane constants: column offset and validity of each row, the y-halo rows, and the
    // x-halo role (left halo of row `lane` for lanes < RY, right halo of row lane - 16 for
    // lanes 16 .. 16 + RY - 1)
    const int b = y0 * nx + x;
    unsigned rows = 0;
#pragma unroll
    for (int r = 0; r < RY; ++r) rows |= (xin && y0 + r < ny) ? 1u << r : 0u;
    const bool lo_ok = xin && y0 >= 1, hi_ok = xin && y0 + RY < ny;
    const int hy = lane < RY ? y0 + lane : (lane >= 16 && lane < 16 + RY) ? y0 + lane - 16 : -1;
    const int hxx = lane < RY ? x0 - 1 : x0 + 32;
    const bool h_ok = hy >= 0 && hy < ny && hxx >= 0 && hxx < nx;
    const int hoff = h_ok ? hy * nx + hxx : 0;
    auto ld = [&](const float *A, int z, bool ok, int off) -> float {
        return (ok && z >= 0 && z < nz) ? A[z * sxy + off] : 0.f;
    };
    float m[RY], cc[RY], p[RY], q[RY];
#pragma unroll
    for (int r = 0; r < RY; ++r) {
        const bool ok = rows >> r & 1u;
        m[r] = ld(Ti, z0 - 1, ok, b + r * nx);
        cc[r] = ld(Ti, z0, ok, b + r * nx);
        p[r] = ld(Ti, z0 + 1, ok, b + r * nx);
        q[r] = ld(QK, z0, ok, b + r * nx);
    }
    float ylo = ld(Ti, z0, lo_ok, b - nx), yhi = ld(Ti, z0, hi_ok, b + RY * nx);
    float hx = ld(Ti, z0, h_ok, hoff);
    for (int z = z0; z < z1; ++z) {
        // loads for the next plane
        float n[RY], qn[RY];
        const bool more = z + 1 < z1;
#pragma unroll
        for (int r = 0; r < RY; ++r) {
            const bool ok = more && (rows >> r & 1u);
            n[r] = ld(Ti, z + 2, ok, b + r * nx);
            qn[r] = ld(QK, z + 1, ok, b + r * nx);
        }
        const float ylon = ld(Ti, z + 1, more && lo_ok, b - nx);
        const float yhin = ld(Ti, z + 1, more && hi_ok, b + RY * nx);
        const float hxn = ld(Ti, z + 1, more && h_ok, hoff);
        const bool zint = z > 0 && z < nz - 1;
        float *out = Tf + z * sxy + b;
#pragma unroll
        for (int r = 0; r < RY; ++r) {
            float xm = __shfl_up_sync(FULL, cc[r], 1), xp = __shfl_down_sync(FULL, cc[r], 1);
            const float hl = __shfl_sync(FULL, hx, r), hr = __shfl_sync(FULL, hx, 16 + r);
            if (lane == 0) xm = hl;
            if (lane == 31) xp = hr;
            const float ym = r == 0 ? ylo : cc[r - 1], yp = r == RY - 1 ? yhi : cc[r + 1];
            if (wint && zint) {
                out[r * nx] = interior_voxel(c, xm, xp, ym, yp, m[r], p[r], q[r]);
            } else if (rows >> r & 1u) {
                float v;
                if (heat_voxel<BC>(c, x, y0 + r, z, nx, ny, nz, xm, xp, ym, yp, m[r], p[r], q[r], v))
                    out[r * nx] = v;
            }
        }
#pragma unroll
        for (int r = 0; r < RY; ++r) {
            m[r] = cc[r];
            cc[r] = p[r];
            p[r] = n[r];
            q[r] = qn[r];
        }
        ylo = ylon;
        yhi = yhin;
        hx = hxn;
    }
}

// Temporal blocking: K sweeps per launch, bit-identical to K single sweeps. A block owns
// a TB_X x TB_Y (x, y) tile and a z chunk of TB_ZC planes; its threads cover the tile with a
// K-voxel halo (one (x, y) column each) and march z as a skewed pipeline: at step p the
// input plane p enters a shared-memory ring (level 0) and level t = 1..K computes plane
// p - 2t from level t-1's planes p-2t-1, p-2t, p-2t+1, all written in earlier steps, so one
// barrier per step suffices (four-plane rings per level). Each level's region shrinks by
// one voxel per side. Every voxel of every level runs heat_voxel, the same float operations
// as a single sweep; voxels the reference never writes keep their value through the levels.
// Q/k enters a 2K-plane ring one step before level 1 needs it. Global loads are issued two
// steps ahead of their use. Global traffic per K sweeps: the input and Q/k with their
// halos, the output once.
constexpr int TB_X = 32, TB_Y = 16, TB_ZC = 50;

template <int K>
struct HeatTB {
    static constexpr int RX = TB_X + 2 * K, RY = TB_Y + 2 * K, RP = RX * RY;
    static constexpr size_t SMEM = (size_t)(4 * K + 2 * K) * RP * sizeof(float);
};

template <int BC, int K>
__global__ void __launch_bounds__(HeatTB<K>::RP, 2) k_heat_tb(float *__restrict__ Tf, const float *__restrict__ Ti,
                                                           const float *__restrict__ QK, const HeatCoef c, int nx,
                                                           int ny, int nz) {
    constexpr int RX = HeatTB<K>::RX, RY = HeatTB<K>::RY, RP = HeatTB<K>::RP;
    extern __shared__ float hsm[];
    float *ring = hsm;              // level t (0..K-1), plane z: ring + (4 t + z % 4) RP
    float *qr = hsm + 4 * K * RP;   // Q/k plane z: qr + (z % 2K) RP
    const int tid = threadIdx.x;
    const int ix = tid % RX, iy = tid / RX;
    const int gx = (int)blockIdx.x * TB_X - K + ix, gy = (int)blockIdx.y * TB_Y - K + iy;
    const bool dom = gx >= 0 && gx < nx && gy >= 0 && gy < ny;
    const bool colint = gx > 0 && gx < nx - 1 && gy > 0 && gy < ny - 1;
    const int z0 = (int)blockIdx.z * TB_ZC, z1 = min(nz, z0 + TB_ZC);
    const size_t sxy = (size_t)nx * ny;
    const float *pT = Ti + (dom ? (size_t)gy * nx + gx : 0);
    const float *pQ = QK + (dom ? (size_t)gy * nx + gx : 0);
    float *pO = Tf + (dom ? (size_t)gy * nx + gx : 0);
    for (int i = tid; i < 6 * K * RP; i += RP) hsm[i] = 0.f;
    const int zlo0 = max(0, z0 - K), zhi0 = min(nz, z1 + K);
    const int qlo = max(0, z0 - K + 1), qhi = min(nz, z1 + K - 1);  // planes level 1 computes
    auto ldT = [&](int z) { return (dom && z >= zlo0 && z < zhi0) ? pT[(size_t)z * sxy] : 0.f; };
    auto ldQ = [&](int z) { return (dom && z >= qlo && z < qhi) ? pQ[(size_t)z * sxy] : 0.f; };
    float t1 = ldT(zlo0), t2 = ldT(zlo0 + 1);
    float q1 = ldQ(zlo0 - 1), q2 = ldQ(zlo0);
    __syncthreads();
    for (int p = zlo0; p < z1 + 2 * K; ++p) {
        // level 0 enters (plane p), Q/k plane p - 1 enters; both are first read next step
        ring[(p & 3) * RP + tid] = t1;
        if (p >= 1) qr[((p - 1) % (2 * K)) * RP + tid] = q1;
        t1 = t2;
        q1 = q2;
        t2 = ldT(p + 2);
        q2 = ldQ(p + 1);
#pragma unroll
        for (int t = 1; t <= K; ++t) {
            const int zt = p - 2 * t;
            const int zlo = max(0, z0 - (K - t)), zhi = min(nz, z1 + (K - t));
            if (zt >= zlo && zt < zhi && dom && ix >= t && ix < RX - t && iy >= t && iy < RY - t) {
                const float *pr = ring + 4 * (t - 1) * RP;
                const float *cur = pr + (zt & 3) * RP;
                const float zm = zt > 0 ? pr[((zt - 1) & 3) * RP + tid] : 0.f;
                const float zp = zt + 1 < nz ? pr[((zt + 1) & 3) * RP + tid] : 0.f;
                float out;
                bool w = true;
                if (colint && zt > 0 && zt < nz - 1)
                    out = interior_voxel(c, cur[tid - 1], cur[tid + 1], cur[tid - RX], cur[tid + RX], zm, zp,
                                         qr[(zt % (2 * K)) * RP + tid]);
                else
                    w = heat_voxel<BC>(c, gx, gy, zt, nx, ny, nz, cur[tid - 1], cur[tid + 1], cur[tid - RX],
                                       cur[tid + RX], zm, zp, qr[(zt % (2 * K)) * RP + tid], out);
                if (t < K)
                    ring[(4 * t + (zt & 3)) * RP + tid] = w ? out : cur[tid];
                else if (w)
                    pO[(size_t)zt * sxy] = out;
            }
        }
        __syncthreads();
    }
}

// sum over voxels of fl((Tf - Ti)^2) accumulated in double (Tfield.h:13-28 sums in float
// sequentially; the stop rule reads this sum rounded to float).
__global__ void k_sq_diff_sum(const float *__restrict__ Tf, const float *__restrict__ Ti, size_t n, double *out) {
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float d = __fsub_rn(Tf[i], Ti[i]);
        acc += (double)__fmul_rn(d, d);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double red[32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = acc;
    __syncthreads();
    if (w == 0) {
        acc = l < (int)(blockDim.x >> 5) ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (l == 0 && acc != 0.0) atomicAdd(out, acc);
    }
}

// out[0] += sum (Tf - Ti)^2, out[1] += sum Tf^2 in FP64 (relative-residual stop rule).
__global__ void k_sq_sums(const float *__restrict__ Tf, const float *__restrict__ Ti, size_t n, double *out) {
    double a[2] = {0.0, 0.0};
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double f = Tf[i], d = f - (double)Ti[i];
        a[0] += d * d;
        a[1] += f * f;
    }
    __shared__ double red[32][2];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int k = 0; k < 2; ++k)
        for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
    if (l == 0) {
        red[w][0] = a[0];
        red[w][1] = a[1];
    }
    __syncthreads();
    if (w == 0) {
        for (int k = 0; k < 2; ++k) {
            double v = l < (int)(blockDim.x >> 5) ? red[l][k] : 0.0;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (l == 0 && v != 0.0) atomicAdd(out + k, v);
        }
    }
}

cudaError_t launch_sq_sums(const float *Tf, const float *Ti, size_t n, double *out2, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out2, 0, 2 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    k_sq_sums<<<1216, 256, 0, st>>>(Tf, Ti, n, out2);
    return cudaGetLastError();
}

// Crystal.h:116-132 in double with no contraction: bit-identical to the host evaluation.
__device__ __forceinline__ float sellmeier_dev(float L, float T) {
    const float A = 4.502483f, B = 0.007294f, C = 0.185087f, D = -0.02357f;
    const float E = 0.073423f, F = 0.199595f, G = 0.001f, H = 7.99724f;
    const double tk = __dadd_rn((double)T, 273.15);
    const double tk2 = __dmul_rn(tk, tk);
    const float b = __double2float_rn(__dmul_rn(3.483933e-8, tk2));
    const float c = __double2float_rn(__dmul_rn(1.607839e-8, tk2));
    const double L2 = __dmul_rn((double)L, (double)L);
    const float Cc = __fadd_rn(C, c), Bb = __fadd_rn(B, b);
    const double t1 = __ddiv_rn((double)Bb, __dsub_rn(L2, __dmul_rn((double)Cc, (double)Cc)));
    const double t2 = __ddiv_rn((double)E, __dsub_rn(L2, __dmul_rn((double)F, (double)F)));
    const double t3 = __ddiv_rn((double)G, __dsub_rn(L2, __dmul_rn((double)H, (double)H)));
    const double t4 = __dmul_rn((double)D, L2);
    const double n2 = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn((double)A, t1), t2), t3), t4);
    return __double2float_rn(__dsqrt_rn(n2));
}

// PPLN index (the congruent LiNbO3 fit of sellmeier_ln, shg_host.cpp) in double with no
// contraction: bit-identical to the host evaluation.
__device__ __forceinline__ float sellmeier_ln_dev(float L, float T) {
    const double a1 = 5.35583, a2 = 0.100473, a3 = 0.20692, a4 = 100.0, a5 = 11.34927, a6 = 1.5334e-2;
    const double b1 = 4.629e-7, b2 = 3.862e-8, b3 = -0.89e-8, b4 = 2.657e-5;
    const double t = (double)T, L2 = __dmul_rn((double)L, (double)L);
    const double f = __dmul_rn(__dsub_rn(t, 24.5), __dadd_rn(t, 570.82));
    const double c3 = __dadd_rn(a3, __dmul_rn(b3, f));
    double n2 = __dadd_rn(a1, __dmul_rn(b1, f));
    n2 = __dadd_rn(n2, __ddiv_rn(__dadd_rn(a2, __dmul_rn(b2, f)), __dsub_rn(L2, __dmul_rn(c3, c3))));
    n2 = __dadd_rn(n2, __ddiv_rn(__dadd_rn(a4, __dmul_rn(b4, f)), __dsub_rn(L2, __dmul_rn(a5, a5))));
    n2 = __dsub_rn(n2, __dmul_rn(a6, L2));
    return __double2float_rn(__dsqrt_rn(n2));
}

// PhaseMatching.h:41-54 per voxel, plus the two indices the thermal z-march needs.
template <int CRYSTAL>
__global__ void k_sellmeier_tables(const float *__restrict__ T, float *NP, float *NS, float *DK, size_t n, float lp,
                                   float ls, float two_pi, float inv_lambda) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float t = T[i];
        const float np = CRYSTAL == 1 ? sellmeier_ln_dev(lp, t) : sellmeier_dev(lp, t);
        const float ns = CRYSTAL == 1 ? sellmeier_ln_dev(ls, t) : sellmeier_dev(ls, t);
        NP[i] = np;
        NS[i] = ns;
        DK[i] = __fmul_rn(two_pi, __fadd_rn(__fsub_rn(__fdiv_rn(__fmul_rn(2.0f, np), lp), __fdiv_rn(ns, ls)), inv_lambda));
    }
}

// ---------------------------------------------------------------------------------------
// Thermal row pass. Stage s of K = nz steps:
//   s == 0        : DKint = DK(slice 0); RK4 of step 0 (slice 0); backward FFT along x;
//   0 < s < nz    : forward FFT; second RK4 of step s-1; heat source of slice s-1;
//                   [capture at s == nz-1]; DKint += DK(slice s); first RK4 of step s;
//                   backward FFT;
//   s == nz       : forward FFT; second RK4 of step nz-1; heat source of slice nz-1.
// The coupling per pixel follows Solver.h:44-63: n from T(x,y,slice), phase
// DKint*(dz*inc + (s+1)*dz)/(s+1) with inc = 0, 0.25, 0.25, 0.5 for the four stages.

__device__ __forceinline__ void block_add_double_th(double v, double *dst) {
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (l == 0 && v != 0.0) atomicAdd(dst, v);
    }
}

// Block shape: LPB lines, one thread per point (LPB * N threads). The row transforms run on
// 2 * LPB * G threads (the pump's lines on the first LPB * G, the SH's on the next), the
// per-point RK4 and heat source on all threads with the point in natural x order, so the
// per-voxel loads are coalesced and the coupling arithmetic is spread over N threads per
// line instead of G.
template <int N>
struct ThRowShape {
    static constexpr int G = LineShape<N>::G;
    static constexpr int LPB = (512 / N < N) ? 512 / N : N;  // lines per block (N = 16: all 16)
    static constexpr int TPB = LPB * N;
    static constexpr int BPI = N / LPB;
    static_assert(LPB >= 1 && N % LPB == 0, "whole lines per block");
    static constexpr int FFT_THREADS = LPB * G;  // per field
    static_assert(FFT_THREADS % 32 == 0 && 2 * FFT_THREADS <= TPB, "transform threads fill whole warps");
};

// The THERMAL row pass for lines [line0, line0 + LPB) at stage s on a block of
// ThRowShape<N>::TPB threads (shared by the streaming launch and the persistent grid).
// Twiddles: the global block g_twiddle + N, or with TS the split's pair table staged in
// shared memory by the caller.
template <int N, bool TS = false>
__device__ __forceinline__ void rows_th_body(const InstDesc &d, const ThermDesc &th, int line0, int s,
                                             float2 *scratch, float2 (*lines)[ThRowShape<N>::LPB * N],
                                             const float2 *tab) {
    using Sh = ThRowShape<N>;
    constexpr int G = Sh::G, E = N / G, LPB = Sh::LPB, FT = Sh::FFT_THREADS;
    constexpr int SC = LineScratch<N, G>::SIZE;
    // stages 0..nz: the THERMAL march runs one stage past the last slice (heat source of slice nz-1)
    if (!SHG_REQUIRE(d.n == N && s >= 0 && s <= th.nz && line0 >= 0 && line0 + LPB <= N, kChkThermalRows, s))
        return;  // block-uniform
    const size_t nxy = (size_t)N * N;
    const int tid = threadIdx.x;
    // transform role: field f, line fl, thread t of the line
    const bool xf = tid < 2 * FT;
    const int f = tid / FT, fl = (tid % FT) / G, t = tid % G;
    float2 *const F = f == 0 ? d.P : d.S;
    float2 *const fline = lines[f & 1] + fl * N;
    float2 *const fsc = scratch + (size_t)((f & 1) * LPB + fl) * SC;
    const size_t fbase = (size_t)(line0 + fl) * N;
    // point role: line l, column x
    const int l = tid / N, x = tid % N;
    const size_t i2 = (size_t)(line0 + l) * N + x;
    float2 *const pP = lines[0] + l * N + x, *const pS = lines[1] + l * N + x;

    if (s == 0) {
        // DKint = DK(slice 0); RK4 of step 0; then the backward transform along x
        float2 vp = d.P[i2], vs = d.S[i2];
        const float dkint = th.DK[i2];
        th.DKint[i2] = dkint;
        const ThCoef k = th_coef(th, th.NP[i2], th.NS[i2], dkint, 0, d.dz);
        rk4_point_th(vp, vs, k, d);
        *pP = vp;
        *pS = vs;
        __syncthreads();
        if (xf) {
            float2 v[E];
#pragma unroll
            for (int j = 0; j < E; ++j) v[j] = fline[t + G * j];
            fft_nat_to_spec<N, G, +1, false, 1, G + 1, TS>(v, t, fsc, tab);
#pragma unroll
            for (int r = 0; r < E; ++r) F[fbase + spec_index<N, G>(t, r)] = v[r];
        }
        return;
    }
    // forward transform of the rows into natural x order
    if (xf) {
        float2 v[E];
#pragma unroll
        for (int j = 0; j < E; ++j) v[j] = F[fbase + t + G * j];
        fft_nat_to_spec<N, G, -1, false, 1, G + 1, TS>(v, t, fsc, tab);
#pragma unroll
        for (int r = 0; r < E; ++r) fline[spec_index<N, G>(t, r)] = v[r];
    }
    __syncthreads();
    const bool capture = (s == th.nz - 1);
    double aS = 0.0, aP = 0.0;
    {
        float2 vp = *pP, vs = *pS;
        const size_t i3 = (size_t)(s - 1) * nxy + i2;
        const float np1 = th.NP[i3], ns1 = th.NS[i3];
        const float dkint = th.DKint[i2];
        const ThCoef k1 = th_coef(th, np1, ns1, dkint, s - 1, d.dz);
        rk4_point_th(vp, vs, k1, d);
        // Tfield.h:277-290: heat source of slice s-1 from the fields after step s-1
        const float a2p = fmaf(vp.x, vp.x, vp.y * vp.y);
        const float a2s = fmaf(vs.x, vs.x, vs.y * vs.y);
        const float Ip = th.qc * np1 * a2p, Is = th.qc * ns1 * a2s;
        const float Q = th.alpha_p * Ip + th.alpha_s * Is + th.beta_s * (Is * Is);
        SHG_AT(th.QK, i3, (size_t)th.nz * nxy, kChkThermalRows) = Q / th.kth;
        if (d.slices && s < th.nz) {
            float2 *sl = d.slices + (size_t)s * 2 * nxy;
            sl[i2] = vp;
            sl[nxy + i2] = vs;
        }
        if (capture) {
            d.Pout[i2] = vp;
            d.Sout[i2] = vs;
            aS = (double)a2s;
            aP = (double)a2p;
        }
        if (s < th.nz) {
            const size_t i3n = (size_t)s * nxy + i2;
            const float dk2 = dkint + th.DK[i3n];
            th.DKint[i2] = dk2;
            const ThCoef k2 = th_coef(th, th.NP[i3n], th.NS[i3n], dk2, s, d.dz);
            rk4_point_th(vp, vs, k2, d);
            *pP = vp;
            *pS = vs;
        } else {
            d.P[i2] = vp;
            d.S[i2] = vs;
        }
    }
    if (capture) {
        block_add_double_th(aS, d.acc + 1);
        block_add_double_th(aP, d.acc + 2);
    }
    if (s == th.nz) return;
    __syncthreads();
    // backward transform along x back to the column pass's layout
    if (xf) {
        float2 v[E];
#pragma unroll
        for (int r = 0; r < E; ++r) v[r] = fline[spec_index<N, G>(t, r)];
        fft_spec_to_nat<N, G, +1, false, 1, G + 1, TS>(v, t, fsc, tab);
#pragma unroll
        for (int j = 0; j < E; ++j) F[fbase + t + G * j] = v[j];
    }
}

template <int N>
__global__ void __launch_bounds__(ThRowShape<N>::TPB) k_rows_th(const InstDesc *__restrict__ dd, const ThermDesc th, int s) {
    using Sh = ThRowShape<N>;
    __shared__ float2 scratch[2 * Sh::LPB * LineScratch<N, Sh::G>::SIZE];
    __shared__ float2 lines[2][Sh::LPB * N];  // [field][line * N + x], natural x order
    rows_th_body<N>(*dd, th, blockIdx.x * Sh::LPB, s, scratch, lines, g_twiddle + N);
}

// Persistent THERMAL march of one solve on a cooperative grid (stages 0..nz): the row pass
// above and the plain column pass (cols_body_h, the same diffraction as k_cols) separated by
// bounded grid-wide barriers instead of kernel boundaries. Block b runs row units b, b + B,
// ... and column groups b + B w (warp w < col_warps), whose propagator values stay in
// registers for the whole run. bar: zeroed arrival counter; err: the solve's error word, or-ed
// with 2 when a barrier wait gave up.
template <int N>
__global__ void __launch_bounds__(ThRowShape<N>::TPB) k_march_coop_th(const InstDesc *__restrict__ dd,
                                                                      const ThermDesc th, unsigned *bar, int *err,
                                                                      int col_warps) {
    using Sh = ThRowShape<N>;
    using C = CoopShape<N>;
    static_assert(C::TPB == Sh::TPB && C::ROW_UNITS == Sh::BPI, "row units are the row pass's blocks");
    constexpr int G = Sh::G;
    __shared__ float2 scratch[2 * Sh::LPB * LineScratch<N, G>::SIZE];
    __shared__ float2 lines[2][Sh::LPB * N];
    __shared__ __align__(16) float2 tws[N];  // the split's twiddle pairs, staged once per launch
    extern __shared__ float2 cscr[];
    const InstDesc &d = *dd;
    if (!SHG_REQUIRE(d.n == N && th.nz >= 1, kChkThermalRows, d.n)) return;  // the whole grid alike
    {
        const float2 *src = twiddle_split<N, G>(g_twiddle + N);
        for (int i = threadIdx.x; i < N; i += blockDim.x) tws[i] = src[i];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int u = blockIdx.x + gridDim.x * warp;
    const bool colw = warp < col_warps && u < C::COL_UNITS;
    const int f = u / (N / C::TC), x = (u % (N / C::TC)) * C::TC + lane % C::TC, t = lane / C::TC;
    float2 h[C::E];
    if (colw) hprop_load<N>(f == 0 ? d.Hp : d.Hs, x, t, h);
    unsigned target = 0;
    for (int s = 0; s <= th.nz; ++s) {
        for (int r = blockIdx.x; r < C::ROW_UNITS; r += gridDim.x) {
            rows_th_body<N, true>(d, th, r * Sh::LPB, s, scratch, lines, tws);
            __syncthreads();  // the block's line buffers are reused by its next unit
        }
        if (s == th.nz) break;
        target += gridDim.x;
        if (!grid_barrier(bar, target, err, 2)) return;
        if (colw) cols_body_h<N, C::TC>(d, x, f, t, cscr + (size_t)warp * C::TC * N + lane % C::TC, h, tws);
        target += gridDim.x;
        if (!grid_barrier(bar, target, err, 2)) return;
    }
}

// ---------------------------------------------------------------------------------------
// Launchers.

cudaError_t launch_init_temperature(float *T, int nx, int ny, int nz, float temp, float t1, float t2, int bc,
                                    cudaStream_t st) {
    k_init_temperature<<<1024, 256, 0, st>>>(T, nx, ny, nz, temp, t1, t2, bc);
    return cudaGetLastError();
}

template <int BC, int K>
static cudaError_t launch_heat_tb_t(float *Tf, const float *Ti, const float *QK, const HeatCoef &c, int nx, int ny,
                                    int nz, cudaStream_t st) {
    static std::atomic<unsigned long long> done{0};  // devices whose shared-memory limit is raised
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 64 || !(done.load() >> dev & 1ull)) {
        e = cudaFuncSetAttribute(k_heat_tb<BC, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)HeatTB<K>::SMEM);
        if (e != cudaSuccess) return e;
        if (dev < 64) done.fetch_or(1ull << dev);
    }
    dim3 grd((nx + TB_X - 1) / TB_X, (ny + TB_Y - 1) / TB_Y, (nz + TB_ZC - 1) / TB_ZC);
    k_heat_tb<BC, K><<<grd, HeatTB<K>::RP, HeatTB<K>::SMEM, st>>>(Tf, Ti, QK, c, nx, ny, nz);
    return cudaGetLastError();
}

int heat_levels() {
    const char *e = std::getenv("SHG_HEAT_TB");
    const int v = e ? std::atoi(e) : 1;
    return (v == 2 || v == 3 || v == 4) ? v : 1;
}

cudaError_t launch_heat_tb(float *Tf, const float *Ti, const float *QK, const HeatCoef &c, int nx, int ny, int nz,
                           int bc, int levels, cudaStream_t st) {
    switch (levels * 2 + (bc != 0)) {
        case 4: return launch_heat_tb_t<0, 2>(Tf, Ti, QK, c, nx, ny, nz, st);
        case 5: return launch_heat_tb_t<1, 2>(Tf, Ti, QK, c, nx, ny, nz, st);
        case 6: return launch_heat_tb_t<0, 3>(Tf, Ti, QK, c, nx, ny, nz, st);
        case 7: return launch_heat_tb_t<1, 3>(Tf, Ti, QK, c, nx, ny, nz, st);
        case 8: return launch_heat_tb_t<0, 4>(Tf, Ti, QK, c, nx, ny, nz, st);
        case 9: return launch_heat_tb_t<1, 4>(Tf, Ti, QK, c, nx, ny, nz, st);
        default: return cudaErrorInvalidValue;
    }
}

// One sweep. SHG_HEAT selects the kernel (all bit-identical):
//   tma   default where the grid allows it (nx a multiple of 4): planes staged by
//         tensor-memory-access copies into a shared-memory ring, 4 tile rows per consumer
//         warp (shg_heat_tma.cu); tma1, tma2, tma8: 1, 2, 8 rows per warp
//   ws4   warp strips of 4 rows, 8 blocks per SM (the default otherwise); ws4b: 6 blocks per
//         SM; ws8: 8-row strips
//   25    2.5D shared-memory tile; simple: one thread per voxel.
// Measured at 256x256x400 on GB300, us per sweep: tma 70.0, tma2 76.1, tma1 92.6, tma8 78.0,
// ws4 96.6, ws4b 100.0, ws8 178, 25 108.6.
cudaError_t launch_heat(float *Tf, const float *Ti, const float *QK, const HeatCoef &c, int nx, int ny, int nz,
                        int bc, int *err, cudaStream_t st) {
    const char *env = std::getenv("SHG_HEAT");
    std::string kind = env ? env : "tma";
    const bool fits32 = (long long)nx * ny * (nz + 3) < (1ll << 31);
    if (kind == "tma" || kind == "tma1" || kind == "tma2" || kind == "tma4" || kind == "tma8") {
        const int rows = kind == "tma" ? 4 : kind[3] - '0';
        if (heat_tma_supported(nx, ny, nz)) return launch_heat_tma(Tf, Ti, QK, c, nx, ny, nz, bc, err, st, rows);
        kind = "ws4";
    }
    if (fits32 && (kind == "ws8" || kind == "ws4" || kind == "ws4b")) {
        const int ry = kind == "ws8" ? 8 : 4, zc = 20;
        dim3 grd((nx + 31) / 32, (ny + ry * WS_WARPS - 1) / (ry * WS_WARPS), (nz + zc - 1) / zc);
        const int blk = 32 * WS_WARPS;
        if (kind == "ws8") {
            if (bc == 0)
                k_heat_ws<0, 8, 4><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz, zc);
            else
                k_heat_ws<1, 8, 4><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz, zc);
        } else if (kind == "ws4") {
            if (bc == 0)
                k_heat_ws<0, 4, 8><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz, zc);
            else
                k_heat_ws<1, 4, 8><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz, zc);
        } else {
            if (bc == 0)
                k_heat_ws<0, 4, 6><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz, zc);
            else
                k_heat_ws<1, 4, 6><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz, zc);
        }
        return cudaGetLastError();
    }
    if (kind != "simple" && fits32) {
        dim3 blk(HT_X, HT_Y, 1);
        dim3 grd((nx + HT_X - 1) / HT_X, (ny + HT_Y - 1) / HT_Y, (nz + HT_Z - 1) / HT_Z);
        if (bc == 0)
            k_heat25<0><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz);
        else
            k_heat25<1><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz);
        return cudaGetLastError();
    }
    dim3 blk(32, 8, 1);
    dim3 grd((nx + 31) / 32, (ny + 7) / 8, nz);
    if (bc == 0)
        k_heat<0><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz);
    else
        k_heat<1><<<grd, blk, 0, st>>>(Tf, Ti, QK, c, nx, ny, nz);
    return cudaGetLastError();
}

cudaError_t launch_sq_diff_sum(const float *Tf, const float *Ti, size_t n, double *out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
    if (e != cudaSuccess) return e;
    k_sq_diff_sum<<<1216, 256, 0, st>>>(Tf, Ti, n, out);
    return cudaGetLastError();
}

cudaError_t launch_sellmeier_tables(const float *T, float *NP, float *NS, float *DK, size_t n, float lp, float ls,
                                    float two_pi, float inv_lambda, int crystal, cudaStream_t st) {
    if (crystal == 1)
        k_sellmeier_tables<1><<<2432, 256, 0, st>>>(T, NP, NS, DK, n, lp, ls, two_pi, inv_lambda);
    else
        k_sellmeier_tables<0><<<2432, 256, 0, st>>>(T, NP, NS, DK, n, lp, ls, two_pi, inv_lambda);
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_rows_th_t(const InstDesc *d, const ThermDesc &th, int s, cudaStream_t st) {
    k_rows_th<N><<<ThRowShape<N>::BPI, ThRowShape<N>::TPB, 0, st>>>(d, th, s);
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_coop_th_t(const InstDesc *d, const ThermDesc &th, unsigned *bar, int *err, cudaStream_t st) {
    using C = CoopShape<N>;
    constexpr int warps = C::TPB / 32;
    auto k = k_march_coop_th<N>;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    // one column group per block where that many blocks fit co-resident, else the fewest
    // blocks that hold every row unit (as for the plain persistent grid)
    int blocks = 0, col_warps = 0;
    size_t smem = 0;
    for (int pass = 0; pass < 2 && !blocks; ++pass) {
        int b = C::ROW_UNITS;
        if (pass == 0 && C::COL_UNITS > b) b = C::COL_UNITS;
        if ((C::COL_UNITS + warps - 1) / warps > b) b = (C::COL_UNITS + warps - 1) / warps;
        const int cw = (C::COL_UNITS + b - 1) / b;
        const size_t sm = (size_t)cw * C::TC * N * sizeof(float2);
        if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, C::TPB, sm)) != cudaSuccess) return e;
        if (per_sm * sms >= b) {
            blocks = b;
            col_warps = cw;
            smem = sm;
        }
    }
    if (!blocks) return cudaErrorCooperativeLaunchTooLarge;
    if (!d) return cudaSuccess;  // fit check only
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks, 1, 1);
    cfg.blockDim = dim3(C::TPB, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, d, th, bar, err, col_warps);
}

cudaError_t launch_coop_th(int n, const InstDesc *d, const ThermDesc &th, unsigned *bar, int *err, cudaStream_t st) {
    switch (n) {
        case 16: return launch_coop_th_t<16>(d, th, bar, err, st);
        case 32: return launch_coop_th_t<32>(d, th, bar, err, st);
        case 64: return launch_coop_th_t<64>(d, th, bar, err, st);
        case 128: return launch_coop_th_t<128>(d, th, bar, err, st);
        case 256: return launch_coop_th_t<256>(d, th, bar, err, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_rows_th(int n, const InstDesc *d, const ThermDesc &th, int s, cudaStream_t st) {
    switch (n) {
        case 16: return launch_rows_th_t<16>(d, th, s, st);
        case 32: return launch_rows_th_t<32>(d, th, s, st);
        case 64: return launch_rows_th_t<64>(d, th, s, st);
        case 128: return launch_rows_th_t<128>(d, th, s, st);
        case 256: return launch_rows_th_t<256>(d, th, s, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace shg
