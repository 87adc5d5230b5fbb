// ORACLE — test infrastructure only. Nothing in the product library links this file.
//
// CPU restatement of the discrete Fourier transform that FFTW3 (fftwf API, version
// unpinned and not vendored by the reference; call sites Solver.h:161-187) computes for
// `fftwf_plan_dft_2d(n0, n1, in, out, sign, flags)`:
//
//     out[i0*n1 + i1] = sum_{j0,j1} in[j0*n1 + j1] * exp(sign * 2*pi*i * (i0*j0/n0 + i1*j1/n1))
//
// unnormalised, row-major n0 x n1, FFTW_FORWARD = -1, FFTW_BACKWARD = +1.
//
// Algorithm: iterative radix-2 decimation-in-time Cooley-Tukey per line (rows, then
// columns through a gathered line buffer), computed in the working precision R
// (float for the fftwf stand-in, double for the FP64 oracle). Twiddles are evaluated in
// double by cos/sin of 2*pi*k/n and rounded once to R; a recurrence would cost ~1e-3 in
// SHG efficiency. Line lengths that are not powers of two fall back to a direct O(n^2)
// DFT with exact (j*k mod n) twiddle indexing, accumulated in double.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

namespace dftref {

template <class R>
struct Line {
    int n = 0;
    bool pow2 = false;
    std::vector<R> twr, twi;      // exp(-2*pi*i*k/n), k < n/2 (pow2) or k < n (direct)
    std::vector<int> rev;         // bit reversal permutation (pow2)
};

template <class R>
const Line<R>& line_tables(int n) {
    static std::mutex mu;
    static std::map<int, std::unique_ptr<Line<R>>> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(n);
    if (it != cache.end()) return *it->second;
    auto L = std::make_unique<Line<R>>();
    L->n = n;
    L->pow2 = n > 0 && (n & (n - 1)) == 0;
    const double two_pi = 6.283185307179586476925286766559;
    int nt = L->pow2 ? (n / 2 > 0 ? n / 2 : 1) : n;
    L->twr.resize(nt);
    L->twi.resize(nt);
    for (int k = 0; k < nt; ++k) {
        double a = two_pi * (double)k / (double)n;
        L->twr[k] = (R)std::cos(a);
        L->twi[k] = (R)(-std::sin(a));
    }
    if (L->pow2) {
        int lg = 0;
        while ((1 << lg) < n) ++lg;
        L->rev.resize(n);
        for (int i = 0; i < n; ++i) {
            int r = 0;
            for (int b = 0; b < lg; ++b)
                if (i & (1 << b)) r |= 1 << (lg - 1 - b);
            L->rev[i] = r;
        }
    }
    auto& ref = *L;
    cache.emplace(n, std::move(L));
    return ref;
}

// In-place transform of one contiguous line of n complex values (re/im interleaved).
template <class R>
void line_dft(R* a, int n, int sign, const Line<R>& T, std::vector<R>& scratch) {
    if (n <= 1) return;
    if (T.pow2) {
        for (int i = 0; i < n; ++i) {
            int r = T.rev[i];
            if (r > i) {
                R tr = a[2 * i], ti = a[2 * i + 1];
                a[2 * i] = a[2 * r];
                a[2 * i + 1] = a[2 * r + 1];
                a[2 * r] = tr;
                a[2 * r + 1] = ti;
            }
        }
        const R sg = (R)(sign < 0 ? 1 : -1);  // table holds exp(-i..); conjugate for sign=+1
        for (int len = 2; len <= n; len <<= 1) {
            int half = len >> 1;
            int step = n / len;
            for (int base = 0; base < n; base += len) {
                for (int k = 0; k < half; ++k) {
                    R wr = T.twr[k * step];
                    R wi = sg * T.twi[k * step];
                    R* u = a + 2 * (base + k);
                    R* v = a + 2 * (base + k + half);
                    R vr = v[0] * wr - v[1] * wi;
                    R vi = v[0] * wi + v[1] * wr;
                    R ur = u[0], ui = u[1];
                    u[0] = ur + vr;
                    u[1] = ui + vi;
                    v[0] = ur - vr;
                    v[1] = ui - vi;
                }
            }
        }
    } else {
        scratch.resize(2 * (size_t)n);
        for (int k = 0; k < n; ++k) {
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < n; ++j) {
                int m = (int)(((int64_t)j * k) % n);
                double wr = (double)T.twr[m];
                double wi = (sign < 0 ? 1.0 : -1.0) * (double)T.twi[m];
                sr += (double)a[2 * j] * wr - (double)a[2 * j + 1] * wi;
                si += (double)a[2 * j] * wi + (double)a[2 * j + 1] * wr;
            }
            scratch[2 * k] = (R)sr;
            scratch[2 * k + 1] = (R)si;
        }
        for (int i = 0; i < 2 * n; ++i) a[i] = scratch[i];
    }
}

// Out-of-place (or in-place when in == out) unnormalised 2D transform over an
// n0 x n1 row-major array of interleaved complex values.
template <class R>
void dft2d(const R* in, R* out, int n0, int n1, int sign) {
    const size_t total = (size_t)n0 * (size_t)n1;
    if (in != out)
        for (size_t i = 0; i < 2 * total; ++i) out[i] = in[i];
    std::vector<R> scratch;
    const Line<R>& T1 = line_tables<R>(n1);
    for (int r = 0; r < n0; ++r) line_dft<R>(out + 2 * (size_t)r * n1, n1, sign, T1, scratch);
    const Line<R>& T0 = line_tables<R>(n0);
    std::vector<R> col(2 * (size_t)n0);
    for (int c = 0; c < n1; ++c) {
        for (int r = 0; r < n0; ++r) {
            col[2 * r] = out[2 * ((size_t)r * n1 + c)];
            col[2 * r + 1] = out[2 * ((size_t)r * n1 + c) + 1];
        }
        line_dft<R>(col.data(), n0, sign, T0, scratch);
        for (int r = 0; r < n0; ++r) {
            out[2 * ((size_t)r * n1 + c)] = col[2 * r];
            out[2 * ((size_t)r * n1 + c) + 1] = col[2 * r + 1];
        }
    }
}

}  // namespace dftref
