// Host side of the GB300 z-march: crystal set-up with the reference's float semantics,
// device memory layout, the batched launch schedule (captured in a CUDA graph), and the
// C ABI declared in include/shg.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <random>
#include <string>
#include <vector>

#include "../../include/shg.h"
#include "shg_internal.h"
#include "shg_march.cuh"
#include "shg_thermal_host.h"
#include "shg_adjoint.h"

#include <memory>

namespace shg {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string &msg) { g_last_error = msg; }

#define SHG_TRY_INT(expr)    \
    do {                     \
        int rc_ = (expr);    \
        if (rc_) return rc_; \
    } while (0)

#define SHG_CUDA(call)                                                                                 \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                            \
            return e_ == cudaErrorMemoryAllocation ? SHG_ERR_NOMEM : SHG_ERR_CUDA;                     \
        }                                                                                              \
    } while (0)

// ---------------------------------------------------------------------------------------
// Crystal set-up. Every expression keeps the reference's operand order and its implicit
// float/double promotions; this file is compiled with -ffp-contract=off.

// Crystal.h:80-82
struct Phys {
    float PI = (float)3.14159265358979323846;
    float C = (float)(299792458 * 1E6 / 1E12);
    float EPS0 = (float)(8.8541878128E-12 * 1E12 / 1E6);
};

// Crystal.h:116-132: float coefficients, double pow/sqrt, float result.
float sellmeier(float L, float T) {
    const float A = 4.502483f, B = 0.007294f, C = 0.185087f, D = -0.02357f;
    const float E = 0.073423f, F = 0.199595f, G = 0.001f, H = 7.99724f;
    const double tk = (double)T + 273.15;
    const float b = (float)(3.483933e-8 * (tk * tk));
    const float c = (float)(1.607839e-8 * (tk * tk));
    const double L2 = (double)L * (double)L;
    const float Cc = C + c, Bb = B + b;
    const double n2 = (double)A + (double)Bb / (L2 - (double)Cc * (double)Cc) +
                      (double)E / (L2 - (double)F * (double)F) + (double)G / (L2 - (double)H * (double)H) +
                      (double)D * L2;
    return (float)std::sqrt(n2);
}

// Extraordinary index of periodically poled lithium niobate (congruent LiNbO3): the
// temperature-dependent Sellmeier fit of D. H. Jundt, Opt. Lett. 22, 1553-1555 (1997),
// L in um, T in C:
//   n^2 = a1 + b1 f + (a2 + b2 f) / (L^2 - (a3 + b3 f)^2) + (a4 + b4 f) / (L^2 - a5^2) - a6 L^2,
//   f = (T - 24.5) (T + 570.82).
// Evaluated in double and rounded to float, like the reference's sPPLT routine. The
// reference's code holds no LiNbO3 routine (its README names an MgO:PPLN crystal), so
// nothing in the reference pins these values; they are the published fit.
float sellmeier_ln(float L, float T) {
    const double a1 = 5.35583, a2 = 0.100473, a3 = 0.20692, a4 = 100.0, a5 = 11.34927, a6 = 1.5334e-2;
    const double b1 = 4.629e-7, b2 = 3.862e-8, b3 = -0.89e-8, b4 = 2.657e-5;
    const double t = (double)T, L2 = (double)L * (double)L;
    const double f = (t - 24.5) * (t + 570.82);
    const double c3 = a3 + b3 * f;
    const double n2 = a1 + b1 * f + (a2 + b2 * f) / (L2 - c3 * c3) + (a4 + b4 * f) / (L2 - a5 * a5) - a6 * L2;
    return (float)std::sqrt(n2);
}

float crystal_index(int crystal, float L, float T) {
    return crystal == SHG_CRYSTAL_PPLN ? sellmeier_ln(L, T) : sellmeier(L, T);
}

// Fill the scalar part of a descriptor (pointers are set by the caller).
void fill_scalars(const shg_config &cr, const SolveParams &sp, InstDesc &d) {
    const Phys ph;
    const float PI = ph.PI;
    const int n = sp.n;
    const float lp = cr.lp, ls = (float)(0.5 * (double)lp);
    const float dx = sp.lx / (float)(unsigned)(n - 1);
    const float dy = sp.ly / (float)(unsigned)(n - 1);
    const float dz = cr.lz / (float)(unsigned)(sp.nz - 1);
    const float dQ = (float)((2.0 / (double)PI) * (double)cr.deff);
    d.n = n;
    d.nz = sp.nz;
    d.nsteps = sp.nz - 1;
    d.dz = dz;
    d.dz6 = dz / 6.0f;
    // Solver.h:75-77: i*pi*dQ/(n_p*lp), i*0.5*pi*dQ/(n_s*ls); TPA and absorption terms.
    const float np_t = crystal_index(cr.crystal, lp, sp.temp), ns_t = crystal_index(cr.crystal, ls, sp.temp);
    d.kp = (dQ * PI) / (np_t * lp);
    d.ks = (dQ * (PI * 0.5f)) / (ns_t * ls);
    d.hp = (float)(0.5 * (double)cr.alpha_p);
    d.tpa0 = (float)(0.5 * (double)cr.alpha_s);
    d.tpa1 = (float)(0.5 * ((double)cr.beta_s * 0.5 * (double)ph.C * (double)ph.EPS0 * (double)ns_t));
    // PhaseMatching.h:57-70
    d.dk = 2.0f * PI * (2.0f * np_t / lp - ns_t / ls + 1.0f / cr.lambda_qpm);
    // Efields.h:74-104 at tpump
    const float np_c = crystal_index(cr.crystal, lp, sp.tpump);
    d.uX = (float)(0.5 * n);
    d.uY = (float)(0.5 * n);
    d.dx = dx;
    d.dy = dy;
    const float wX2 = sp.waist * sp.waist;
    const float zRX = PI * np_c * wX2 / lp;
    const float Ap0 = sqrtf(4.0f * sp.power / (ph.EPS0 * ph.C * PI * np_c * wX2));
    const float etaX = sp.focal / zRX;
    const float mre = 1.0f - etaX * 0.0f, mim = -(etaX * 1.0f);
    const float mden = mre * mre + mim * mim;
    d.amp = make_float2((+Ap0 * mre) / mden, (-Ap0 * mim) / mden);
    d.wM = make_float2(wX2 * mre, wX2 * mim);
    d.wM_den = d.wM.x * d.wM.x + d.wM.y * d.wM.y;
    // Efields.h:107-126 at tprop
    const float np_h = crystal_index(cr.crystal, lp, sp.tprop), ns_h = crystal_index(cr.crystal, ls, sp.tprop);
    const float kpw = 2.0f * PI * np_h / lp, ksw = 2.0f * PI * ns_h / ls;
    const float dfX = 1.0f / dx / (float)(unsigned)n, dfY = 1.0f / dy / (float)(unsigned)n;
    const float pi2 = PI * PI;
    d.gp = 2.0f * pi2 / kpw;
    d.gs = 2.0f * pi2 / ksw;
    d.dfX2 = dfX * dfX;
    d.dfY2 = dfY * dfY;
    d.linp = 2.0f * PI * dfX * tanf(cr.rho_p);
    d.lins = 2.0f * PI * dfX * tanf(cr.rho_s);
    d.mdz = -dz;
    d.inv_nn = 1.0f / (float)(n * n);
}

// Power of a field in W from sum |A|^2 (the efficiency definition used by the tests).
double field_power(double sum_abs2, float n_index, float dx, float dy) {
    const Phys ph;
    return 0.5 * (double)ph.EPS0 * (double)ph.C * (double)n_index * sum_abs2 * (double)dx * (double)dy;
}

// SHG_ERR_NOMEM, checked on the host, when `bytes` exceed the free memory of the current
// device: a request that cannot fit is refused before it reaches the allocator.
int device_fits(size_t bytes, const char *what) {
    size_t free_b = 0, total_b = 0;
    SHG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (bytes > free_b) {
        set_error(std::string(what) + ": needs " + std::to_string(bytes >> 20) + " MiB of device memory, " +
                  std::to_string(free_b >> 20) + " MiB free");
        return SHG_ERR_NOMEM;
    }
    return SHG_OK;
}

// Inter-stage twiddle tables of the line FFTs (layout at g_twiddle in shg_fft.cuh): for
// N = 16..256 and the splits G = line_threads(N) (at [N, 2N)) and G / 2 for N >= 64 (at
// [2*kMaxLine + N, 2*kMaxLine + 2N)), float2 2*(j*G + t) + b holds w_N^(t*(2j + b)),
// w_N^m = exp(-2 pi i m/N) evaluated in double and rounded once.
int ensure_twiddles(int device) {
    static std::mutex mu;
    static std::map<int, bool> done;
    std::lock_guard<std::mutex> lock(mu);
    if (done[device]) return SHG_OK;
    std::vector<float2> tab(4 * kMaxLine, make_float2(0.f, 0.f));
    for (int N = 16; N <= kMaxLine; N *= 2) {
        auto w = [N](int m) {
            const double a = 2.0 * 3.14159265358979323846264338327950288 * (double)(m % N) / (double)N;
            return make_float2((float)std::cos(a), (float)(-std::sin(a)));
        };
        for (int split = 0; split < (N >= 64 ? 2 : 1); ++split) {
            const int G = line_threads(N) >> split, E = N / G;
            float2 *dst = tab.data() + split * 2 * kMaxLine + N;
            for (int j = 0; j < E / 2; ++j)
                for (int t = 0; t < G; ++t) {
                    dst[2 * (j * G + t)] = w(t * 2 * j);
                    dst[2 * (j * G + t) + 1] = w(t * (2 * j + 1));
                }
        }
    }
    for (const float2 *addr : {twiddle_symbol_address_march(), twiddle_symbol_address_thermal(),
                               twiddle_symbol_address_adjoint(), twiddle_symbol_address_resident(),
                               twiddle_symbol_address_resident128(), twiddle_symbol_address_resident256(),
                               twiddle_symbol_address_cluster_pt()}) {
        void *p = const_cast<float2 *>(addr);
        if (!p) {
            set_error("twiddle table symbol unavailable");
            return SHG_ERR_CUDA;
        }
        SHG_CUDA(cudaMemcpy(p, tab.data(), tab.size() * sizeof(float2), cudaMemcpyHostToDevice));
    }
    done[device] = true;
    return SHG_OK;
}

// Name of a class schedule: "streaming", "coop" (persistent grid), "cluster" (one cluster
// per solve, one thread per point) or "cs/minb/g".
std::string schedule_label(bool resident, const ResidentVariant &v) {
    if (!resident) return "streaming";
    if (v.cs == 0) return "coop";
    if (v.cs == -1) return "cluster";
    return std::to_string(v.cs) + "/" + std::to_string(v.minb) + "/" + std::to_string(v.g);
}

// ---------------------------------------------------------------------------------------
// A set of plain solves with their device buffers and launch schedule.
class Batch {
   public:
    ~Batch() {
        release();
        for (auto s2 : side_streams_) cudaStreamDestroy(s2);
        for (auto e2 : side_events_) cudaEventDestroy(e2);
        if (fork_event_) cudaEventDestroy(fork_event_);
    }

    int create(const shg_config &crystal, const std::vector<SolveParams> &sp) {
        release();
        cr_ = crystal;
        sp_ = sp;
        const int n = (int)sp.size();
        if (n <= 0) {
            set_error("empty batch");
            return SHG_ERR_INVALID;
        }
        for (const auto &s : sp) {
            if (!line_length_supported(s.n)) {
                set_error("grid " + std::to_string(s.n) + " not supported (square power of two in [16, 256])");
                return SHG_ERR_UNSUPPORTED;
            }
            if (s.nz < 2) {
                set_error("nz must be >= 2");
                return SHG_ERR_INVALID;
            }
        }
        SHG_CUDA(cudaSetDevice(crystal.device));
        int rc = ensure_twiddles(crystal.device);
        if (rc) return rc;
        // Memory plan: six regions (P, S, Pout, Sout, Hp, Hs), each holding the n*n complex
        // points of every solve back to back in solve order (so a region is one contiguous
        // copy), then the per-slice constants (nz float4 per solve) and the sums (4 doubles
        // per solve). Each solve's block is a multiple of 2 KiB, so every pointer stays
        // 256-byte aligned.
        auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
        foff_.assign(n + 1, 0);
        size_t nz_total = 0;
        for (int i = 0; i < n; ++i) {
            foff_[i + 1] = foff_[i] + (size_t)sp[i].n * sp[i].n;
            nz_total += (size_t)sp[i].nz;
        }
        const size_t pts = foff_[n];
        const size_t region = al(pts * sizeof(float2));
        const size_t step_off = 6 * region;
        const size_t acc_off = step_off + al(nz_total * sizeof(float4));
        const size_t total = acc_off + al(4 * sizeof(double) * n);
        SHG_TRY_INT(device_fits(total, "batch"));
        SHG_CUDA(cudaMalloc(&pool_, total));
        pool_bytes_ = total;
        acc_ = reinterpret_cast<double *>(pool_ + acc_off);
        desc_.resize(n);
        p_src_.assign(n, nullptr);
        s_src_.assign(n, nullptr);
        max_nn_ = 0;
        max_nz_ = 0;
        size_t zoff = 0;
        for (int i = 0; i < n; ++i) {
            InstDesc &d = desc_[i];
            std::memset(&d, 0, sizeof(d));
            const size_t nn = (size_t)sp[i].n * sp[i].n;
            auto reg = [&](int r) { return reinterpret_cast<float2 *>(pool_ + r * region) + foff_[i]; };
            d.P = reg(0);
            d.S = reg(1);
            d.Pout = reg(2);
            d.Sout = reg(3);
            d.Hp = reg(4);
            d.Hs = reg(5);
            d.stepc = reinterpret_cast<float4 *>(pool_ + step_off) + zoff;
            zoff += (size_t)sp[i].nz;
            d.acc = acc_ + 4 * i;
            fill_scalars(cr_, sp[i], d);
            max_nn_ = std::max(max_nn_, (int)nn);
            max_nz_ = std::max(max_nz_, sp[i].nz);
        }
        sout_all_ = desc_[0].Sout;
        SHG_CUDA(cudaMalloc(&d_desc_, n * sizeof(InstDesc)));
        // Size classes, each sorted by step count (descending) so that the solves still
        // marching at stage s form a prefix of the class list.
        std::map<int, std::vector<int>> by_n;
        for (int i = 0; i < n; ++i) by_n[sp[i].n].push_back(i);
        std::vector<int> lists;
        classes_.clear();
        for (auto &kv : by_n) {
            auto &v = kv.second;
            std::stable_sort(v.begin(), v.end(), [&](int a, int b) { return desc_[a].nsteps > desc_[b].nsteps; });
            Class c;
            c.n = kv.first;
            c.offset = (int)lists.size();
            c.count = (int)v.size();
            for (int i : v) {
                lists.push_back(i);
                c.steps.push_back(desc_[i].nsteps);
            }
            classes_.push_back(c);
        }
        // schedule per class from SHG_MARCH: "auto" (default: the autotuner picks at the first
        // run), "streaming", "resident" (default variants), or a list "n:streaming" /
        // "n:cs/minb" / "n:coop" / "n:cluster" per grid (e.g. "64:1/1,128:4/2,256:16/2";
        // unlisted grids: autotuner; "coop", the persistent cooperative grid, applies to a
        // batch of one solve; "cluster" runs each solve in one cluster of the cluster march)
        const char *mode = std::getenv("SHG_MARCH");
        const std::string m = mode ? mode : "auto";
        for (auto &c : classes_) {
            for (int k = 0; k < c.count; ++k) c.pt_steps += (double)c.n * c.n * c.steps[k];
            c.tuned = m == "streaming" || m == "resident";
            c.resident = m != "streaming";
            if (c.resident) c.var = resident_default(c.n);
            const std::string key = std::to_string(c.n) + ":";
            for (size_t pos = 0; pos < m.size();) {
                size_t end = m.find(',', pos);
                if (end == std::string::npos) end = m.size();
                const std::string item = m.substr(pos, end - pos);
                pos = end + 1;
                if (item.compare(0, key.size(), key) != 0) continue;
                const std::string v = item.substr(key.size());
                int cs = 0, mb = 0, g = 0;
                if (v == "streaming") {
                    c.resident = false;
                    c.tuned = true;
                } else if (v == "coop") {
                    if (classes_.size() == 1 && c.count == 1) {
                        c.resident = true;
                        c.var = ResidentVariant{0, 0, 0};
                        c.tuned = true;
                    }
                } else if (v == "cluster") {
                    if (cluster_pt_size(c.n) > 0) {
                        c.resident = true;
                        c.var = ResidentVariant{-1, 1, 0};
                        c.tuned = true;
                    }
                } else if (std::sscanf(v.c_str(), "%d/%d/%d", &cs, &mb, &g) >= 2) {
                    ResidentVariant vs[16];
                    const int nv = resident_variants(c.n, vs, 16);
                    for (int i = nv - 1; i >= 0; --i)
                        if (vs[i].cs == cs && vs[i].minb == mb && (g == 0 || vs[i].g == g)) {
                            c.resident = true;
                            c.var = vs[i];
                            c.tuned = true;
                        }
                }
            }
            if (c.resident) SHG_CUDA(prepare_resident(c.n, c.var, &c.max_clusters));
        }
        // resident march: class streams (largest solves first) and one job counter per class
        while ((int)side_streams_.size() < (int)classes_.size()) {
            cudaStream_t s2;
            SHG_CUDA(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
            side_streams_.push_back(s2);
            cudaEvent_t e2;
            SHG_CUDA(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming));
            side_events_.push_back(e2);
        }
        if (!fork_event_) SHG_CUDA(cudaEventCreateWithFlags(&fork_event_, cudaEventDisableTiming));
        SHG_CUDA(cudaMalloc(&d_counters_, 64 * sizeof(int)));
        SHG_CUDA(cudaMalloc(&d_lists_, lists.size() * sizeof(int)));
        SHG_CUDA(cudaMemcpy(d_lists_, lists.data(), lists.size() * sizeof(int), cudaMemcpyHostToDevice));
        SHG_CUDA(cudaMemset(pool_, 0, pool_bytes_));
        desc_dirty_ = true;
        return SHG_OK;
    }

    // Replace the crystal constants (grid fields ignored) and refresh every descriptor.
    void set_crystal(const shg_config &c) {
        const int nx = cr_.nx, ny = cr_.ny, nz = cr_.nz, dev = cr_.device;
        const float lx = cr_.lx, ly = cr_.ly;
        cr_ = c;
        cr_.nx = nx;
        cr_.ny = ny;
        cr_.nz = nz;
        cr_.lx = lx;
        cr_.ly = ly;
        cr_.device = dev;
        for (int i = 0; i < (int)desc_.size(); ++i) {
            const int keep_given = desc_[i].pump_given;
            fill_scalars(cr_, sp_[i], desc_[i]);
            desc_[i].pump_given = keep_given;
        }
        desc_dirty_ = true;
    }

    // Re-parameterise solve i (same grid) without reallocating.
    int set_params(int i, const SolveParams &sp) {
        if (i < 0 || i >= (int)desc_.size() || sp.n != sp_[i].n || sp.nz != sp_[i].nz) {
            set_error("set_params: grid change needs a new handle");
            return SHG_ERR_INVALID;
        }
        sp_[i] = sp;
        const int keep_given = desc_[i].pump_given;
        fill_scalars(cr_, sp, desc_[i]);
        desc_[i].pump_given = keep_given;
        desc_dirty_ = true;  // the graph reads descriptors from device memory: no re-capture
        return SHG_OK;
    }

    // Per-slice capture buffer of solve i (nullptr: off); slot 0 receives the input state.
    void set_slices(int i, float2 *slices) {
        if (desc_[i].slices != slices) {
            desc_[i].slices = slices;
            desc_dirty_ = true;
            invalidate_graph();
        }
    }

    // Device buffers copied into P / S at the start of every run (nullptr: Gaussian pump
    // built on the device / SH cleared to zero).
    void set_sources(int i, const float2 *p_src, const float2 *s_src) {
        if (p_src_[i] != p_src || s_src_[i] != s_src) {
            p_src_[i] = p_src;
            s_src_[i] = s_src;
            invalidate_graph();
        }
        const int given = p_src ? 1 : 0;
        if (desc_[i].pump_given != given) {
            desc_[i].pump_given = given;
            desc_dirty_ = true;
            invalidate_graph();
        }
    }

    // Enqueue set-up and the march for every solve on `st` (a CUDA graph after the
    // first call when use_graph is set).
    int run_async(cudaStream_t st, bool use_graph) {
        SHG_TRY_INT(tune(st));
        if (desc_dirty_) {
            SHG_CUDA(cudaMemcpyAsync(d_desc_, desc_.data(), desc_.size() * sizeof(InstDesc), cudaMemcpyHostToDevice, st));
            desc_dirty_ = false;
        }
        if (!use_graph) return enqueue(st);
        if (!graph_exec_) {
            // Capture on a private stream (the caller's may be the legacy default stream,
            // which cannot be captured); the graph is then launched on the caller's stream.
            if (!capture_stream_) SHG_CUDA(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking));
            cudaGraph_t g = nullptr;
            SHG_CUDA(cudaStreamBeginCapture(capture_stream_, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue(capture_stream_);
            cudaError_t e = cudaStreamEndCapture(capture_stream_, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            SHG_CUDA(e);
            e = cudaGraphInstantiate(&graph_exec_, g, 0);
            cudaGraphDestroy(g);
            SHG_CUDA(e);
        }
        SHG_CUDA(cudaGraphLaunch(graph_exec_, st));
        return SHG_OK;
    }

    // The persistent cooperative grid is offered only to a batch of one solve: it holds every
    // SM it is given, so it never shares the device with another class's side stream.
    bool lone_solve() const { return classes_.size() == 1 && classes_[0].count == 1; }

    int launch_count() const {
        int c = 2;  // set-up kernels
        for (const auto &k : classes_) {
            const int K = k.steps.empty() ? 0 : k.steps[0];
            c += k.resident ? 1 : (K + 1) + K;
        }
        return c;
    }

    // Autotuner: for every class not yet scheduled, time the streaming schedule and each
    // resident variant on the class's own solves (set-up included in every trial, the
    // second of two runs counted) and keep the fastest. Choices are cached per device and
    // class shape (grid, solve count, step total) for the life of the process.
    int tune(cudaStream_t st) {
        bool any = false;
        for (auto &c : classes_) any |= !c.tuned;
        if (!any) return SHG_OK;
        if (desc_dirty_) {
            SHG_CUDA(cudaMemcpyAsync(d_desc_, desc_.data(), desc_.size() * sizeof(InstDesc), cudaMemcpyHostToDevice, st));
            desc_dirty_ = false;
        }
        static std::mutex mu;
        static std::map<std::tuple<int, int, int, double, bool>, std::pair<bool, ResidentVariant>> cache;
        cudaEvent_t a, b;
        SHG_CUDA(cudaEventCreate(&a));
        SHG_CUDA(cudaEventCreate(&b));
        int rc = SHG_OK;
        for (int ci = 0; ci < (int)classes_.size() && rc == SHG_OK; ++ci) {
            Class &c = classes_[ci];
            if (c.tuned) continue;
            const auto key = std::make_tuple(cr_.device, c.n, c.count, c.pt_steps, lone_solve());
            {
                std::lock_guard<std::mutex> lock(mu);
                auto it = cache.find(key);
                if (it != cache.end()) {
                    c.resident = it->second.first;
                    c.var = it->second.second;
                    if (c.resident) rc = prepare_resident(c.n, c.var, &c.max_clusters) == cudaSuccess ? SHG_OK : SHG_ERR_CUDA;
                    c.tuned = true;
                    continue;
                }
            }
            struct Cand {
                bool resident;
                ResidentVariant v;
                int clusters;
            };
            std::vector<Cand> cands{{false, {0, 0, 0}, 0}};
            ResidentVariant vs[16];
            const int nv = resident_variants(c.n, vs, 16);
            for (int i = 0; i < nv; ++i) {
                int mc = 0;
                if (prepare_resident(c.n, vs[i], &mc) == cudaSuccess && mc > 0)
                    cands.push_back({true, vs[i], mc});
                else
                    cudaGetLastError();  // a variant that does not fit is skipped
            }
            if (cluster_pt_size(c.n) > 0) {  // one cluster per solve, where the class fits in one wave
                int mc = 0;
                if (prepare_resident(c.n, ResidentVariant{-1, 1, 0}, &mc) == cudaSuccess && mc >= c.count)
                    cands.push_back({true, ResidentVariant{-1, 1, 0}, mc});
                else
                    cudaGetLastError();
            }
            if (lone_solve()) {  // one solve in the batch: the persistent cooperative grid as well
                int mc = 0;
                if (prepare_resident(c.n, ResidentVariant{0, 0, 0}, &mc) == cudaSuccess && mc > 0)
                    cands.push_back({true, ResidentVariant{0, 0, 0}, 1});
                else
                    cudaGetLastError();
            }
            float best = 1e30f;
            int bi = 0;
            c.trials.clear();
            for (int i = 0; i < (int)cands.size() && rc == SHG_OK; ++i) {
                c.resident = cands[i].resident;
                c.var = cands[i].v;
                c.max_clusters = cands[i].clusters;
                float ms = 0.f;
                for (int rep = 0; rep < 2 && rc == SHG_OK; ++rep) {
                    rc = enqueue_inputs(st);
                    if (rc) break;
                    if (launch_setup(d_desc_, (int)desc_.size(), max_nn_, max_nz_, st) != cudaSuccess ||
                        cudaMemsetAsync(d_counters_, 0, 64 * sizeof(int), st) != cudaSuccess ||
                        cudaEventRecord(a, st) != cudaSuccess) {
                        rc = SHG_ERR_CUDA;
                        break;
                    }
                    rc = enqueue_class(ci, st, nullptr);
                    if (rc) break;
                    if (cudaEventRecord(b, st) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
                        cudaEventElapsedTime(&ms, a, b) != cudaSuccess)
                        rc = SHG_ERR_CUDA;
                }
                c.trials.push_back({cands[i].resident, cands[i].v, ms});
                if (ms < best) {
                    best = ms;
                    bi = i;
                }
            }
            if (rc) break;
            c.resident = cands[bi].resident;
            c.var = cands[bi].v;
            c.max_clusters = cands[bi].clusters;
            c.tuned = true;
            std::lock_guard<std::mutex> lock(mu);
            cache[key] = {c.resident, c.var};
        }
        if (rc == SHG_OK) rc = tune_mix(st, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if (rc && rc != SHG_ERR_CUDA) return rc;
        if (rc) {
            set_error("autotune: CUDA error while timing a schedule");
            return rc;
        }
        invalidate_graph();
        return SHG_OK;
    }

    // Second stage: the classes share the GPU in a run (one stream each), so the fastest
    // schedule of a class alone is not always the fastest beside the others. For each class
    // the two fastest schedules alone (and the streaming passes for classes of one to three
    // solves) are tried, timing the whole concurrent run of every combination as a captured
    // graph (second of two launches). Also run for a single class, whose first-stage times
    // come from direct launches. Cached per device and batch shape.
    int tune_mix(cudaStream_t st, cudaEvent_t a, cudaEvent_t b) {
        const int nc = (int)classes_.size();
        mix_.clear();
        if (nc < 1) return SHG_OK;
        std::vector<int> order(nc);
        for (int i = 0; i < nc; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](int x, int y) { return classes_[x].n > classes_[y].n; });
        std::string key = std::to_string(cr_.device);
        for (int ci : order) {
            char buf[96];
            std::snprintf(buf, sizeof(buf), "|%d:%d:%.17g", classes_[ci].n, classes_[ci].count, classes_[ci].pt_steps);
            key += buf;
        }
        struct Pick {
            bool resident;
            ResidentVariant v;
        };
        static std::mutex mu;
        static std::map<std::string, std::vector<Pick>> cache;
        auto apply = [&](int ci, const Pick &p) -> int {
            Class &c = classes_[ci];
            c.resident = p.resident;
            c.var = p.v;
            if (c.resident && prepare_resident(c.n, c.var, &c.max_clusters) != cudaSuccess) {
                cudaGetLastError();
                return SHG_ERR_CUDA;
            }
            return SHG_OK;
        };
        {
            std::lock_guard<std::mutex> lock(mu);
            auto it = cache.find(key);
            if (it != cache.end()) {
                for (int oi = 0; oi < nc; ++oi) SHG_TRY_INT(apply(order[oi], it->second[oi]));
                return SHG_OK;
            }
        }
        std::vector<std::vector<Pick>> opts(nc);
        int ncomb = 1;
        for (int oi = 0; oi < nc; ++oi) {
            auto t = classes_[order[oi]].trials;
            if (t.empty()) return SHG_OK;  // schedule fixed by the caller: keep it
            std::sort(t.begin(), t.end(), [](const Trial &x, const Trial &y) { return x.ms < y.ms; });
            for (int k = 0; k < (int)t.size() && k < 2; ++k) opts[oi].push_back({t[k].resident, t[k].v});
            // a class of one to three solves: the first stage times direct launches, where
            // the streaming passes (two small launches per step) pay the host's launch cost
            // that a captured graph does not, so they are always timed here as well
            bool has_streaming = false;
            for (const Pick &p : opts[oi]) has_streaming |= !p.resident;
            if (classes_[order[oi]].count < 4 && !has_streaming) opts[oi].push_back({false, {0, 0, 0}});
            ncomb *= (int)opts[oi].size();
        }
        float best = 1e30f;
        int bi = 0;
        for (int comb = 0; comb < ncomb; ++comb) {
            int r = comb;
            std::string label;
            for (int oi = 0; oi < nc; ++oi) {
                const int k = r % (int)opts[oi].size();
                r /= (int)opts[oi].size();
                const Pick &p = opts[oi][k];
                SHG_TRY_INT(apply(order[oi], p));
                label += (oi ? "," : "") + std::to_string(classes_[order[oi]].n) + ":" + schedule_label(p.resident, p.v);
            }
            // time the combination as runs execute it: a captured graph, second launch counted
            float ms = 0.f;
            invalidate_graph();
            SHG_TRY_INT(run_async(st, true));
            if (cudaEventRecord(a, st) != cudaSuccess) return SHG_ERR_CUDA;
            SHG_TRY_INT(run_async(st, true));
            if (cudaEventRecord(b, st) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
                cudaEventElapsedTime(&ms, a, b) != cudaSuccess)
                return SHG_ERR_CUDA;
            mix_.push_back({label, ms});
            if (ms < best) {
                best = ms;
                bi = comb;
            }
        }
        std::vector<Pick> chosen(nc);
        int r = bi;
        for (int oi = 0; oi < nc; ++oi) {
            const int k = r % (int)opts[oi].size();
            r /= (int)opts[oi].size();
            chosen[oi] = opts[oi][k];
            SHG_TRY_INT(apply(order[oi], chosen[oi]));
        }
        std::lock_guard<std::mutex> lock(mu);
        cache[key] = chosen;
        return SHG_OK;
    }

    // Fixes the schedule of grid-size class n: streaming (resident = 0) or the resident
    // variant (cs, minb), which must be one of resident_variants(n) and fit on the device.
    int set_schedule(int n, int resident, int cs, int minb, int g = 0) {
        for (auto &c : classes_) {
            if (c.n != n) continue;
            if (!resident) {
                c.resident = false;
            } else if (resident == 2) {
                int mc = 0;
                if (!lone_solve() || prepare_resident(n, ResidentVariant{0, 0, 0}, &mc) != cudaSuccess || mc < 1) {
                    cudaGetLastError();
                    set_error("set_schedule: the persistent grid runs a batch of one solve whose grid fits co-resident");
                    return SHG_ERR_UNSUPPORTED;
                }
                c.resident = true;
                c.var = ResidentVariant{0, 0, 0};
                c.max_clusters = 1;
            } else if (resident == 3) {
                int mc = 0;
                if (cluster_pt_size(n) < 1 || prepare_resident(n, ResidentVariant{-1, 1, 0}, &mc) != cudaSuccess ||
                    mc < 1) {
                    cudaGetLastError();
                    set_error("set_schedule: the cluster march runs grids 64, 128 and 256 where a cluster fits");
                    return SHG_ERR_UNSUPPORTED;
                }
                c.resident = true;
                c.var = ResidentVariant{-1, 1, 0};
                c.max_clusters = mc;
            } else {
                ResidentVariant vs[16];
                const int nv = resident_variants(n, vs, 16);
                int hit = -1;
                for (int i = nv - 1; i >= 0; --i)
                    if (vs[i].cs == cs && vs[i].minb == minb && (g == 0 || vs[i].g == g)) hit = i;
                int mc = 0;
                if (hit < 0 || prepare_resident(n, vs[hit], &mc) != cudaSuccess || mc < 1) {
                    cudaGetLastError();
                    set_error("set_schedule: no such resident variant for this grid, or it does not fit");
                    return SHG_ERR_UNSUPPORTED;
                }
                c.resident = true;
                c.var = vs[hit];
                c.max_clusters = mc;
            }
            c.tuned = true;
            invalidate_graph();
            return SHG_OK;
        }
        set_error("set_schedule: no class with that grid size");
        return SHG_ERR_INVALID;
    }

    // Concurrent run of the march as enqueue() launches it (classes on side streams, no
    // graph) with events around each class: start / end of every class in ms after the
    // common start, in class order.
    int timeline(cudaStream_t st, std::vector<double> &se) {
        SHG_TRY_INT(tune(st));
        if (desc_dirty_) {
            SHG_CUDA(cudaMemcpyAsync(d_desc_, desc_.data(), desc_.size() * sizeof(InstDesc), cudaMemcpyHostToDevice, st));
            desc_dirty_ = false;
        }
        SHG_TRY_INT(enqueue_inputs(st));
        SHG_CUDA(launch_setup(d_desc_, (int)desc_.size(), max_nn_, max_nz_, st));
        SHG_CUDA(cudaMemsetAsync(d_counters_, 0, 64 * sizeof(int), st));
        const int nc = (int)classes_.size();
        std::vector<cudaEvent_t> ev(2 * nc + 1);
        for (auto &e : ev) SHG_CUDA(cudaEventCreate(&e));
        SHG_CUDA(cudaEventRecord(ev[0], st));
        for (int ci = 0; ci < nc; ++ci) {
            cudaStream_t ss = side_streams_[ci];
            SHG_CUDA(cudaStreamWaitEvent(ss, ev[0], 0));
            SHG_CUDA(cudaEventRecord(ev[1 + 2 * ci], ss));
            SHG_TRY_INT(enqueue_class(ci, ss, nullptr));
            SHG_CUDA(cudaEventRecord(ev[2 + 2 * ci], ss));
        }
        for (int ci = 0; ci < nc; ++ci) SHG_CUDA(cudaStreamWaitEvent(st, ev[2 + 2 * ci], 0));
        SHG_CUDA(cudaStreamSynchronize(st));
        se.assign(2 * nc, 0.0);
        for (int i = 0; i < 2 * nc; ++i) {
            float ms = 0.f;
            SHG_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1 + i]));
            se[i] = ms;
        }
        for (auto &e : ev) cudaEventDestroy(e);
        return SHG_OK;
    }

    // One line per class: grid, solves, chosen schedule and the trial times (ms).
    std::string schedule() const {
        std::string out;
        for (const auto &c : classes_) {
            out += "n=" + std::to_string(c.n) + " solves=" + std::to_string(c.count) + ": ";
            out += !c.tuned                      ? std::string("untuned")
                   : !c.resident                   ? std::string("streaming")
                   : c.var.cs == 0                 ? std::string("coop (persistent grid)")
                   : c.var.cs == -1                ? std::string("cluster march")
                                                   : "resident cs=" + std::to_string(c.var.cs) + " minb=" +
                                                       std::to_string(c.var.minb) + " g=" + std::to_string(c.var.g);
            if (!c.trials.empty()) {
                out += " [";
                for (size_t i = 0; i < c.trials.size(); ++i) {
                    const auto &t = c.trials[i];
                    char buf[96];
                    std::snprintf(buf, sizeof(buf), "%s%s %.3f", i ? ", " : "", schedule_label(t.resident, t.v).c_str(),
                                  t.ms);
                    out += buf;
                }
                out += " ms]";
            }
            out += "\n";
        }
        if (!mix_.empty()) {
            out += "concurrent run:";
            for (const auto &m : mix_) {
                char buf[160];
                std::snprintf(buf, sizeof(buf), " [%s %.3f ms]", m.first.c_str(), m.second);
                out += buf;
            }
            out += "\n";
        }
        return out;
    }

    int copy_acc(std::vector<double> &acc) {
        acc.resize(4 * desc_.size());
        SHG_CUDA(cudaMemcpy(acc.data(), acc_, acc.size() * sizeof(double), cudaMemcpyDeviceToHost));
        return check_run_errors();
    }

    // Error word of the last run (set when a grid-barrier wait of the persistent grid gave up);
    // read after the run has completed.
    int check_run_errors() {
        int flag = 0;
        SHG_CUDA(cudaMemcpy(&flag, d_counters_ + 63, sizeof(int), cudaMemcpyDeviceToHost));
        if (flag) {
            set_error("persistent grid: a grid-barrier wait gave up (run incomplete)");
            return SHG_ERR_CUDA;
        }
        return SHG_OK;
    }

    // Efficiency of solve i from accumulated sums.
    double eta_of(int i, const std::vector<double> &acc) const {
        const SolveParams &s = sp_[i];
        const float dx = desc_[i].dx, dy = desc_[i].dy;
        const float np_c = crystal_index(cr_.crystal, cr_.lp, s.temp),
                    ns_c = crystal_index(cr_.crystal, (float)(0.5 * (double)cr_.lp), s.temp);
        const double pin = field_power(acc[4 * i + 0], np_c, dx, dy);
        const double psh = field_power(acc[4 * i + 1], ns_c, dx, dy);
        return psh / pin;
    }

    void powers_of(int i, const std::vector<double> &acc, double *pin, double *psh, double *pout) const {
        const SolveParams &s = sp_[i];
        const float dx = desc_[i].dx, dy = desc_[i].dy;
        const float np_c = crystal_index(cr_.crystal, cr_.lp, s.temp),
                    ns_c = crystal_index(cr_.crystal, (float)(0.5 * (double)cr_.lp), s.temp);
        if (pin) *pin = field_power(acc[4 * i + 0], np_c, dx, dy);
        if (psh) *psh = field_power(acc[4 * i + 1], ns_c, dx, dy);
        if (pout) *pout = field_power(acc[4 * i + 2], np_c, dx, dy);
    }

    const InstDesc &desc(int i) const { return desc_[i]; }
    // SH output fields of all solves, contiguous in solve order; offset of solve i in points.
    const float2 *sout_all() const { return sout_all_; }
    const float2 *pout_all() const { return desc_[0].Pout; }
    size_t field_offset(int i) const { return foff_[i]; }
    size_t total_points() const { return foff_.back(); }
    int size() const { return (int)desc_.size(); }
    const SolveParams &params(int i) const { return sp_[i]; }

   private:
    struct Trial {
        bool resident;
        ResidentVariant v;
        float ms;
    };
    struct Class {
        int n = 0, offset = 0, count = 0;
        std::vector<int> steps;  // descending
        bool tuned = false;      // schedule chosen (by SHG_MARCH or the autotuner)
        bool resident = true;    // resident march (else streaming row / column launches)
        ResidentVariant var{1, 1, 0};
        int max_clusters = 0;    // resident march: clusters resident at once
        double pt_steps = 0;     // sum of n*n*nsteps
        std::vector<Trial> trials;
    };

   public:
    // Per-launch timing of one un-captured run: events around every kernel launch.
    struct Recorder {
        struct Rec {
            std::string name;
            double bytes;
            cudaEvent_t a, b;
        };
        std::vector<Rec> recs;
        int begin(const std::string &name, double bytes, cudaStream_t st) {
            Rec r{name, bytes, nullptr, nullptr};
            SHG_CUDA(cudaEventCreate(&r.a));
            SHG_CUDA(cudaEventCreate(&r.b));
            SHG_CUDA(cudaEventRecord(r.a, st));
            recs.push_back(r);
            return SHG_OK;
        }
        int end(cudaStream_t st) {
            SHG_CUDA(cudaEventRecord(recs.back().b, st));
            return SHG_OK;
        }
        ~Recorder() {
            for (auto &r : recs) {
                if (r.a) cudaEventDestroy(r.a);
                if (r.b) cudaEventDestroy(r.b);
            }
        }
    };

    int profile(cudaStream_t st, Recorder &rec) {
        SHG_TRY_INT(tune(st));
        if (desc_dirty_) {
            SHG_CUDA(cudaMemcpyAsync(d_desc_, desc_.data(), desc_.size() * sizeof(InstDesc), cudaMemcpyHostToDevice, st));
            desc_dirty_ = false;
        }
        SHG_TRY_INT(enqueue(st, &rec));
        SHG_CUDA(cudaStreamSynchronize(st));
        return SHG_OK;
    }

    // Upload descriptors, place the input fields and run only the set-up kernels
    // (propagators, step constants, input power): the state the adjoint starts from.
    int setup_only(cudaStream_t st) {
        if (desc_dirty_) {
            SHG_CUDA(cudaMemcpyAsync(d_desc_, desc_.data(), desc_.size() * sizeof(InstDesc), cudaMemcpyHostToDevice, st));
            desc_dirty_ = false;
        }
        SHG_TRY_INT(enqueue_inputs(st));
        SHG_CUDA(launch_setup(d_desc_, (int)desc_.size(), max_nn_, max_nz_, st));
        return SHG_OK;
    }

    const InstDesc *device_desc() const { return d_desc_; }

   private:
    int enqueue_inputs(cudaStream_t st) {
        SHG_CUDA(cudaMemsetAsync(acc_, 0, 4 * sizeof(double) * desc_.size(), st));
        for (int i = 0; i < (int)desc_.size(); ++i) {
            const size_t bytes = (size_t)desc_[i].n * desc_[i].n * sizeof(float2);
            if (p_src_[i]) SHG_CUDA(cudaMemcpyAsync(desc_[i].P, p_src_[i], bytes, cudaMemcpyDeviceToDevice, st));
            if (s_src_[i])
                SHG_CUDA(cudaMemcpyAsync(desc_[i].S, s_src_[i], bytes, cudaMemcpyDeviceToDevice, st));
            else
                SHG_CUDA(cudaMemsetAsync(desc_[i].S, 0, bytes, st));
        }
        return SHG_OK;
    }

    int enqueue(cudaStream_t st, Recorder *rec = nullptr) {
        SHG_CUDA(cudaMemsetAsync(acc_, 0, 4 * sizeof(double) * desc_.size(), st));
        for (int i = 0; i < (int)desc_.size(); ++i) {
            const size_t bytes = (size_t)desc_[i].n * desc_[i].n * sizeof(float2);
            if (p_src_[i]) SHG_CUDA(cudaMemcpyAsync(desc_[i].P, p_src_[i], bytes, cudaMemcpyDeviceToDevice, st));
            if (s_src_[i])
                SHG_CUDA(cudaMemcpyAsync(desc_[i].S, s_src_[i], bytes, cudaMemcpyDeviceToDevice, st));
            else
                SHG_CUDA(cudaMemsetAsync(desc_[i].S, 0, bytes, st));
        }
        if (rec) SHG_TRY_INT(rec->begin("setup", 24.0 * (double)total_points(), st));
        SHG_CUDA(launch_setup(d_desc_, (int)desc_.size(), max_nn_, max_nz_, st));
        if (rec) SHG_TRY_INT(rec->end(st));
        for (int i = 0; i < (int)desc_.size(); ++i)
            if (desc_[i].slices) {
                const size_t nn = (size_t)desc_[i].n * desc_[i].n;
                SHG_CUDA(cudaMemcpyAsync(desc_[i].slices, desc_[i].P, nn * sizeof(float2), cudaMemcpyDeviceToDevice, st));
                SHG_CUDA(cudaMemcpyAsync(desc_[i].slices + nn, desc_[i].S, nn * sizeof(float2),
                                         cudaMemcpyDeviceToDevice, st));
            }
        SHG_CUDA(cudaMemsetAsync(d_counters_, 0, 64 * sizeof(int), st));
        // classes in descending grid size; concurrently on side streams unless timed
        std::vector<int> order(classes_.size());
        for (int i = 0; i < (int)order.size(); ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](int x, int y) { return classes_[x].n > classes_[y].n; });
        if (rec || order.size() == 1) {
            for (int ci : order) SHG_TRY_INT(enqueue_class(ci, st, rec));
            return SHG_OK;
        }
        SHG_CUDA(cudaEventRecord(fork_event_, st));
        for (int oi = 0; oi < (int)order.size(); ++oi) {
            cudaStream_t ss = side_streams_[oi];
            SHG_CUDA(cudaStreamWaitEvent(ss, fork_event_, 0));
            SHG_TRY_INT(enqueue_class(order[oi], ss, nullptr));
            SHG_CUDA(cudaEventRecord(side_events_[oi], ss));
        }
        for (int oi = 0; oi < (int)order.size(); ++oi) SHG_CUDA(cudaStreamWaitEvent(st, side_events_[oi], 0));
        return SHG_OK;
    }

    // The march of class ci on `st` with its current schedule.
    int enqueue_class(int ci, cudaStream_t st, Recorder *rec) {
        const Class &k = classes_[ci];
        const int *list = d_lists_ + k.offset;
        if (k.resident && k.var.cs == 0) {
            // the persistent cooperative grid of a lone solve: barrier words 40 + 2 ci, error word 63
            unsigned *bar = reinterpret_cast<unsigned *>(d_counters_ + 40 + 2 * ci);
            if (rec) SHG_TRY_INT(rec->begin("coop<" + std::to_string(k.n) + ">", 32.0 * k.pt_steps, st));
            SHG_CUDA(launch_coop(k.n, d_desc_, list, bar, d_counters_ + 63, st));
            if (rec) SHG_TRY_INT(rec->end(st));
            return SHG_OK;
        }
        if (k.resident) {
            int *counter = d_counters_ + ci;
            const char *kind = k.var.cs == -1 ? "cluster<" : "resident<";
            if (rec) SHG_TRY_INT(rec->begin(kind + std::to_string(k.n) + ">", 32.0 * k.pt_steps, st));
            SHG_CUDA(launch_resident(k.n, k.var, d_desc_, list, k.count, counter, k.max_clusters, st));
            if (rec) SHG_TRY_INT(rec->end(st));
            return SHG_OK;
        }
        const int K = k.steps[0];
        const double nn = (double)k.n * k.n;
        const std::string rn = "rows<" + std::to_string(k.n) + ">", cn = "cols<" + std::to_string(k.n) + ">";
        for (int s = 0; s <= K; ++s) {
            // solves with nsteps >= s run the row pass, nsteps >= s + 1 the column pass
            const int nr = count_at_least(k.steps, s), nc = count_at_least(k.steps, s + 1);
            // algorithmic bytes: both fields read and written (rows), plus both
            // propagators read (columns)
            if (rec) SHG_TRY_INT(rec->begin(rn, 32.0 * nn * nr, st));
            SHG_CUDA(launch_rows(k.n, d_desc_, list, nr, s, st));
            if (rec) SHG_TRY_INT(rec->end(st));
            if (nc > 0) {
                if (rec) SHG_TRY_INT(rec->begin(cn, 48.0 * nn * nc, st));
                SHG_CUDA(launch_cols(k.n, d_desc_, list, nc, st));
                if (rec) SHG_TRY_INT(rec->end(st));
            }
        }
        return SHG_OK;
    }

    static int count_at_least(const std::vector<int> &desc_sorted, int v) {
        // desc_sorted is descending: count of entries >= v
        int lo = 0, hi = (int)desc_sorted.size();
        while (lo < hi) {
            const int mid = (lo + hi) / 2;
            if (desc_sorted[mid] >= v)
                lo = mid + 1;
            else
                hi = mid;
        }
        return lo;
    }

    void invalidate_graph() {
        if (graph_exec_) {
            cudaGraphExecDestroy(graph_exec_);
            graph_exec_ = nullptr;
        }
    }

    void release() {
        invalidate_graph();
        if (d_counters_) cudaFree(d_counters_);
        d_counters_ = nullptr;
        if (capture_stream_) cudaStreamDestroy(capture_stream_);
        capture_stream_ = nullptr;
        if (pool_) cudaFree(pool_);
        if (d_desc_) cudaFree(d_desc_);
        if (d_lists_) cudaFree(d_lists_);
        pool_ = nullptr;
        d_desc_ = nullptr;
        d_lists_ = nullptr;
    }

    shg_config cr_{};
    std::vector<SolveParams> sp_;
    std::vector<InstDesc> desc_;
    std::vector<size_t> foff_;
    const float2 *sout_all_ = nullptr;
    std::vector<const float2 *> p_src_, s_src_;
    std::vector<Class> classes_;
    char *pool_ = nullptr;
    size_t pool_bytes_ = 0;
    double *acc_ = nullptr;
    InstDesc *d_desc_ = nullptr;
    int *d_lists_ = nullptr;
    int max_nn_ = 0, max_nz_ = 0;
    bool desc_dirty_ = true;
    cudaGraphExec_t graph_exec_ = nullptr;
    cudaStream_t capture_stream_ = nullptr;
    int *d_counters_ = nullptr;
    std::vector<std::pair<std::string, float>> mix_;  // concurrent-run trials of the autotuner
    std::vector<cudaStream_t> side_streams_;
    std::vector<cudaEvent_t> side_events_;
    cudaEvent_t fork_event_ = nullptr;
};

int validate_config(const shg_config &c) {
    if (c.crystal != SHG_CRYSTAL_SPPLT && c.crystal != SHG_CRYSTAL_PPLN) {
        set_error("crystal must be SHG_CRYSTAL_SPPLT or SHG_CRYSTAL_PPLN");
        return SHG_ERR_INVALID;
    }
    if (c.nx <= 1 || c.ny <= 1 || c.nz <= 1) {
        set_error("grid sizes must be > 1");
        return SHG_ERR_INVALID;
    }
    if (!(c.lx > 0) || !(c.ly > 0) || !(c.lz > 0) || !(c.lp > 0) || !(c.lambda_qpm != 0)) {
        set_error("window, crystal length, wavelength and poling period must be positive");
        return SHG_ERR_INVALID;
    }
    if (c.nx != c.ny || !line_length_supported(c.nx)) {
        set_error("the device path needs a square grid with NX = NY a power of two in [16, 256]");
        return SHG_ERR_UNSUPPORTED;
    }
    return SHG_OK;
}

}  // namespace shg

using namespace shg;

struct shg_handle {
    shg_config cfg;
    Batch batch;
    std::unique_ptr<ThermalSolve> th;  // set for thermal configurations
    std::unique_ptr<AdjointWork> adj;  // work space of gradient passes
    std::string out_dir;               // Files.h outputs of shg_run when set
    float2 *slices = nullptr;          // per-slice states for save_only_last = 0
    SolveParams sp{};
    int n = 0;
    float2 *stage_p = nullptr, *stage_s = nullptr;  // device staging of given input fields
    bool pump_given = false, sh_given = false, have_pump = false, have_result = false;
    cudaStream_t stream = nullptr;
    ~shg_handle() {
        if (slices) cudaFree(slices);
        if (stage_p) cudaFree(stage_p);
        if (stage_s) cudaFree(stage_s);
        if (stream) cudaStreamDestroy(stream);
    }
};

struct shg_batch {
    shg_config cfg;
    Batch batch;
    cudaStream_t stream = nullptr;
    bool ran = false;
    ~shg_batch() {
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// Efields.h:129-144 with a fixed seed: std::default_random_engine and
// std::normal_distribution<float>(0, 1e-20), two draws per point (re, im).
void noise_field(unsigned seed, size_t n, std::vector<float2> &out) {
    std::default_random_engine generator(seed);
    std::normal_distribution<float> distribution(0.0, 1.0e-20);
    out.resize(n);
    for (size_t i = 0; i < n; ++i) {
        const float a1 = distribution(generator);
        const float a2 = distribution(generator);
        out[i] = make_float2(a1, a2);
    }
}

int handle_run(shg_handle *h, cudaStream_t st) {
    Batch &b = h->batch;
    int rc = b.set_params(0, h->sp);
    if (rc) return rc;
    b.set_sources(0, h->pump_given ? h->stage_p : nullptr, h->sh_given ? h->stage_s : nullptr);
    rc = b.run_async(st, true);
    if (rc) return rc;
    h->have_result = true;
    return SHG_OK;
}

// Solver.h:250-262 and :340 outputs: Pump_out/Signal_out (top of slice NZ-1) or
// Pump_<s>/Signal_<s> for every slice, and Tfinal_<z> when requested (THERMAL).
int write_outputs(shg_handle *h, bool save_only_last, bool save_temperature) {
    const int n = h->n, nz = h->cfg.nz;
    const size_t nn = (size_t)n * n;
    std::vector<float2> a(nn), b(nn);
    if (save_only_last) {
        SHG_TRY_INT(shg_get_fields(h, reinterpret_cast<float *>(a.data()), reinterpret_cast<float *>(b.data())));
        if (!save_matrix_complex(h->out_dir, "Pump_out", a.data(), n, n) ||
            !save_matrix_complex(h->out_dir, "Signal_out", b.data(), n, n)) {
            set_error("cannot write output files in " + h->out_dir);
            return SHG_ERR_INVALID;
        }
    } else {
        std::vector<float2> all((size_t)nz * 2 * nn);
        SHG_CUDA(cudaMemcpy(all.data(), h->slices, all.size() * sizeof(float2), cudaMemcpyDeviceToHost));
        for (int s = 0; s < nz; ++s) {
            const float2 *st = all.data() + (size_t)s * 2 * nn;
            if (!save_matrix_complex(h->out_dir, "Pump_" + std::to_string(s), st, n, n) ||
                !save_matrix_complex(h->out_dir, "Signal_" + std::to_string(s), st + nn, n, n)) {
                set_error("cannot write output files in " + h->out_dir);
                return SHG_ERR_INVALID;
            }
        }
    }
    if (save_temperature && h->th) {
        std::vector<float> T(nn * (size_t)nz);
        SHG_TRY_INT(h->th->copy_temperature(T.data()));
        if (!save_tensor_real(h->out_dir, "Tfinal", T.data(), n, n, nz)) {
            set_error("cannot write Tfinal files in " + h->out_dir);
            return SHG_ERR_INVALID;
        }
    }
    return SHG_OK;
}

int check_handle(shg_handle *h) {
    if (!h) {
        set_error("null handle");
        return SHG_ERR_INVALID;
    }
    return SHG_OK;
}

}  // namespace

#define SHG_TRY(expr)          \
    do {                       \
        int rc_ = (expr);      \
        if (rc_) return rc_;   \
    } while (0)

extern "C" {

int shg_config_init(shg_config *c) {
    if (!c) {
        set_error("null config");
        return SHG_ERR_INVALID;
    }
    std::memset(c, 0, sizeof(*c));
    c->nx = 64;
    c->ny = 64;
    c->nz = 200;
    c->lx = 2000.0f;
    c->ly = 1000.0f;
    c->lz = 30000.0f;
    c->lp = 1.064f;
    c->deff = 11.00e-6f;
    c->lambda_qpm = 7.97f;
    c->alpha_p = 0.17e-6f;
    c->alpha_s = 1.57e-6f;
    c->beta_s = 5e-5f;
    c->rho_p = 0.0f;
    c->rho_s = 0.0f;
    c->kth = 8.4e-6f;
    c->htc = 10e-12f;
    c->thermal = 0;
    c->bc = 0;
    c->sh_seed = -1;
    c->device = 0;
    c->crystal = SHG_CRYSTAL_SPPLT;
    return SHG_OK;
}

int shg_index(int crystal, float lambda_um, float temp_c, float *n) {
    if (!n || (crystal != SHG_CRYSTAL_SPPLT && crystal != SHG_CRYSTAL_PPLN) || !(lambda_um > 0)) {
        set_error("shg_index: unknown crystal, non-positive wavelength or null output");
        return SHG_ERR_INVALID;
    }
    *n = crystal_index(crystal, lambda_um, temp_c);
    if (!std::isfinite(*n)) {
        set_error("shg_index: the index is not finite at this wavelength and temperature");
        return SHG_ERR_NONFINITE;
    }
    return SHG_OK;
}

const char *shg_last_error(void) { return g_last_error.c_str(); }

int shg_create(const shg_config *cfg, shg_handle **out) {
    if (!cfg || !out) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    *out = nullptr;
    SHG_TRY(validate_config(*cfg));
    auto *h = new shg_handle;
    h->cfg = *cfg;
    h->n = cfg->nx;
    if (cfg->thermal) {
        if (cfg->bc != 0 && cfg->bc != 1) {
            delete h;
            set_error("bc must be 0 (open top) or 1 (oven surrounded)");
            return SHG_ERR_INVALID;
        }
        h->th.reset(new ThermalSolve);
        int rc = h->th->create(*cfg);
        if (rc) {
            delete h;
            return rc;
        }
        *out = h;
        return SHG_OK;
    }
    h->sp = SolveParams{cfg->nx, cfg->nz, cfg->lx, cfg->ly, 1.0f, 30.0f, 0.5f * cfg->lz, 50.0f, 50.0f, 50.0f};
    int rc = h->batch.create(*cfg, {h->sp});
    if (rc) {
        delete h;
        return rc;
    }
    const size_t bytes = (size_t)h->n * h->n * sizeof(float2);
    if (cudaMalloc(&h->stage_p, bytes) != cudaSuccess || cudaMalloc(&h->stage_s, bytes) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("device allocation for the handle failed");
        delete h;
        return SHG_ERR_NOMEM;
    }
    *out = h;
    return SHG_OK;
}

int shg_destroy(shg_handle *h) {
    delete h;
    return SHG_OK;
}

int shg_set_input_pump(shg_handle *h, float power, float focalpoint, float waist, float tc) {
    SHG_TRY(check_handle(h));
    if (h->th) {
        set_error("plain-path entry point called on a thermal handle");
        return SHG_ERR_STATE;
    }
    h->sp.power = power;
    h->sp.focal = focalpoint;
    h->sp.waist = waist;
    h->sp.tpump = tc;
    h->pump_given = false;
    h->have_pump = true;
    return SHG_OK;
}

int shg_set_input_fields(shg_handle *h, const float *pump, const float *sh) {
    SHG_TRY(check_handle(h));
    if (h->th) {
        set_error("plain-path entry point called on a thermal handle");
        return SHG_ERR_STATE;
    }
    if (!pump) {
        set_error("pump field required");
        return SHG_ERR_INVALID;
    }
    const size_t bytes = (size_t)h->n * h->n * sizeof(float2);
    SHG_CUDA(cudaMemcpy(h->stage_p, pump, bytes, cudaMemcpyHostToDevice));
    h->pump_given = true;
    h->have_pump = true;
    if (sh) {
        SHG_CUDA(cudaMemcpy(h->stage_s, sh, bytes, cudaMemcpyHostToDevice));
        h->sh_given = true;
    } else {
        h->sh_given = false;
    }
    return SHG_OK;
}

int shg_cwes(shg_handle *h, float temp) {
    shg::Phase phase("shg_cwes");
    SHG_TRY(check_handle(h));
    if (h->th) {
        set_error("plain-path entry point called on a thermal handle");
        return SHG_ERR_STATE;
    }
    if (!h->have_pump) {
        set_error("shg_cwes: no input pump (shg_set_input_pump or shg_set_input_fields first)");
        return SHG_ERR_STATE;
    }
    h->sp.temp = temp;
    h->sp.tprop = temp;
    SHG_TRY(handle_run(h, h->stream));
    SHG_CUDA(cudaStreamSynchronize(h->stream));
    if (!h->th) SHG_TRY(h->batch.check_run_errors());
    return SHG_OK;
}

int shg_cwes_device(shg_handle *h, float temp, const void *pump_in, const void *sh_in, void *pump_out,
                    void *sh_out, void *stream) {
    shg::Phase phase("shg_cwes_device");
    SHG_TRY(check_handle(h));
    if (h->th) {
        set_error("plain-path entry point called on a thermal handle");
        return SHG_ERR_STATE;
    }
    if (!pump_in) {
        set_error("pump_in required");
        return SHG_ERR_INVALID;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t bytes = (size_t)h->n * h->n * sizeof(float2);
    SHG_CUDA(cudaMemcpyAsync(h->stage_p, pump_in, bytes, cudaMemcpyDeviceToDevice, st));
    if (sh_in) SHG_CUDA(cudaMemcpyAsync(h->stage_s, sh_in, bytes, cudaMemcpyDeviceToDevice, st));
    h->pump_given = true;
    h->sh_given = sh_in != nullptr;
    h->have_pump = true;
    h->sp.temp = temp;
    h->sp.tprop = temp;
    SHG_TRY(handle_run(h, st));
    const InstDesc &d = h->batch.desc(0);
    if (pump_out) SHG_CUDA(cudaMemcpyAsync(pump_out, d.Pout, bytes, cudaMemcpyDeviceToDevice, st));
    if (sh_out) SHG_CUDA(cudaMemcpyAsync(sh_out, d.Sout, bytes, cudaMemcpyDeviceToDevice, st));
    return SHG_OK;
}

int shg_run(shg_handle *h, float power, float waist, float focalpoint, float temp, float t_inf, float t_peltier1,
            float t_peltier2, int save_only_last, int save_temperature) {
    shg::Phase phase("shg_run");
    SHG_TRY(check_handle(h));
    (void)save_only_last;
    (void)save_temperature;
    if (h->th) {
        const bool per_slice = !h->out_dir.empty() && !save_only_last;
        if (per_slice && !h->slices)
            SHG_CUDA(cudaMalloc(&h->slices, (size_t)h->cfg.nz * 2 * h->n * h->n * sizeof(float2)));
        h->th->set_slices(per_slice ? h->slices : nullptr);
        SHG_TRY(h->th->run(power, waist, focalpoint, temp, t_inf, t_peltier1, t_peltier2));
        h->have_result = true;
        if (!h->out_dir.empty()) SHG_TRY(write_outputs(h, save_only_last, save_temperature));
        return SHG_OK;
    }
    // Solver.h:342-348: pump, SH start, propagators and delta-k all at Temp.
    h->sp.power = power;
    h->sp.waist = waist;
    h->sp.focal = focalpoint;
    h->sp.temp = temp;
    h->sp.tpump = temp;
    h->sp.tprop = temp;
    h->pump_given = false;
    h->have_pump = true;
    if (h->cfg.sh_seed >= 0) {
        std::vector<float2> nz;
        noise_field((unsigned)h->cfg.sh_seed, (size_t)h->n * h->n, nz);
        SHG_CUDA(cudaMemcpy(h->stage_s, nz.data(), nz.size() * sizeof(float2), cudaMemcpyHostToDevice));
        h->sh_given = true;
    } else {
        h->sh_given = false;
    }
    const bool per_slice = !h->out_dir.empty() && !save_only_last;
    if (per_slice && !h->slices)
        SHG_CUDA(cudaMalloc(&h->slices, (size_t)h->cfg.nz * 2 * h->n * h->n * sizeof(float2)));
    h->batch.set_slices(0, per_slice ? h->slices : nullptr);
    SHG_TRY(handle_run(h, h->stream));
    SHG_CUDA(cudaStreamSynchronize(h->stream));
    if (!h->th) SHG_TRY(h->batch.check_run_errors());
    if (!h->out_dir.empty()) SHG_TRY(write_outputs(h, save_only_last, false));
    return SHG_OK;
}

int shg_get_fields(shg_handle *h, float *pump_out, float *sh_out) {
    SHG_TRY(check_handle(h));
    if (!h->have_result) {
        set_error("no result yet");
        return SHG_ERR_STATE;
    }
    if (h->th) return h->th->copy_fields(pump_out, sh_out);
    const InstDesc &d = h->batch.desc(0);
    const size_t bytes = (size_t)h->n * h->n * sizeof(float2);
    SHG_CUDA(cudaStreamSynchronize(h->stream));
    SHG_TRY(h->batch.check_run_errors());
    if (pump_out) SHG_CUDA(cudaMemcpy(pump_out, d.Pout, bytes, cudaMemcpyDeviceToHost));
    if (sh_out) SHG_CUDA(cudaMemcpy(sh_out, d.Sout, bytes, cudaMemcpyDeviceToHost));
    return SHG_OK;
}

int shg_get_powers(shg_handle *h, double *p_pump_in, double *p_sh_out, double *p_pump_out) {
    SHG_TRY(check_handle(h));
    if (!h->have_result) {
        set_error("no result yet");
        return SHG_ERR_STATE;
    }
    if (h->th) return h->th->powers(p_pump_in, p_sh_out, p_pump_out);
    std::vector<double> acc;
    // the run was enqueued on the handle's stream (shg_run / shg_cwes) or the caller's
    // (shg_cwes_device, which the caller orders before this call): waiting for the
    // handle's stream leaves every other handle and stream on the device running
    SHG_CUDA(cudaStreamSynchronize(h->stream));
    SHG_TRY(h->batch.copy_acc(acc));
    h->batch.powers_of(0, acc, p_pump_in, p_sh_out, p_pump_out);
    return SHG_OK;
}

int shg_efficiency(shg_handle *h, double *eta) {
    double pin = 0, psh = 0;
    SHG_TRY(shg_get_powers(h, &pin, &psh, nullptr));
    *eta = psh / pin;
    if (!std::isfinite(*eta)) {
        set_error("efficiency is not finite");
        return SHG_ERR_NONFINITE;
    }
    return SHG_OK;
}

int shg_grad_device(shg_handle *h, float temp, const void *pump_in, const void *sh_in, int checkpoints,
                    void *grad_pump, void *grad_sh, double *out4, void *stream) {
    shg::Phase phase("shg_grad_device");
    SHG_TRY(check_handle(h));
    if (h->th) {
        set_error("shg_grad_device: gradients are for plain handles (hold the temperature field fixed)");
        return SHG_ERR_STATE;
    }
    if (!pump_in || !out4) {
        set_error("shg_grad_device: pump_in and out4 are required");
        return SHG_ERR_INVALID;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t bytes = (size_t)h->n * h->n * sizeof(float2);
    SHG_CUDA(cudaMemcpyAsync(h->stage_p, pump_in, bytes, cudaMemcpyDeviceToDevice, st));
    if (sh_in) SHG_CUDA(cudaMemcpyAsync(h->stage_s, sh_in, bytes, cudaMemcpyDeviceToDevice, st));
    h->pump_given = true;
    h->sh_given = sh_in != nullptr;
    h->have_pump = true;
    h->sp.temp = temp;
    h->sp.tprop = temp;
    SHG_TRY(h->batch.set_params(0, h->sp));
    h->batch.set_sources(0, h->stage_p, h->sh_given ? h->stage_s : nullptr);
    SHG_TRY(h->batch.setup_only(st));
    if (!h->adj) h->adj.reset(new AdjointWork);
    return adjoint_run(h->cfg, h->batch.desc(0), h->batch.device_desc(), temp, checkpoints, *h->adj, st,
                       static_cast<float2 *>(grad_pump), static_cast<float2 *>(grad_sh), out4);
}

int shg_grad_run(shg_handle *h, float power, float waist, float focalpoint, float temp, const void *pump_factor,
                 int checkpoints, void *grad_pump, double *out8, void *stream) {
    shg::Phase phase("shg_grad_run");
    SHG_TRY(check_handle(h));
    if (h->th) {
        set_error("shg_grad_run: gradients are for plain handles (hold the temperature field fixed)");
        return SHG_ERR_STATE;
    }
    if (!out8) {
        set_error("shg_grad_run: out8 is required");
        return SHG_ERR_INVALID;
    }
    if (!(power > 0) || !(waist > 0) || !std::isfinite(focalpoint) || !std::isfinite(temp)) {
        set_error("shg_grad_run: power and waist must be positive, focal point and temperature finite");
        return SHG_ERR_INVALID;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // Solver.h:342-348: pump (setPump at Temp), propagators and delta-k at Temp, SH from zero
    h->sp.power = power;
    h->sp.waist = waist;
    h->sp.focal = focalpoint;
    h->sp.temp = temp;
    h->sp.tpump = temp;
    h->sp.tprop = temp;
    h->pump_given = false;
    h->sh_given = false;
    h->have_pump = true;
    SHG_TRY(h->batch.set_params(0, h->sp));
    h->batch.set_slices(0, nullptr);
    h->batch.set_sources(0, nullptr, nullptr);
    SHG_TRY(h->batch.setup_only(st));
    const InstDesc &d = h->batch.desc(0);
    const float2 *factor = static_cast<const float2 *>(pump_factor);
    if (factor) SHG_CUDA(launch_cmul_inplace(d.P, factor, h->n * h->n, st));
    if (!h->adj) h->adj.reset(new AdjointWork);
    SHG_TRY(adjoint_run(h->cfg, d, h->batch.device_desc(), temp, checkpoints, *h->adj, st,
                        static_cast<float2 *>(grad_pump), nullptr, out8));
    double pg[4];
    SHG_TRY(pump_param_gradients(h->cfg, d, power, waist, focalpoint, temp, factor, *h->adj, st, pg));
    out8[4] = pg[0];
    out8[5] = pg[1];
    out8[6] = pg[2];
    out8[7] = out8[1] + pg[3];
    return SHG_OK;
}

int shg_set_output_dir(shg_handle *h, const char *dir) {
    SHG_TRY(check_handle(h));
    h->out_dir = dir ? dir : "";
    return SHG_OK;
}

int shg_set_poling_period(shg_handle *h, float lambda_qpm) {
    SHG_TRY(check_handle(h));
    if (!(lambda_qpm != 0.0f) || !std::isfinite(lambda_qpm)) {
        set_error("poling period must be finite and non-zero");
        return SHG_ERR_INVALID;
    }
    h->cfg.lambda_qpm = lambda_qpm;
    if (h->th) {
        set_error("shg_set_poling_period: not for thermal handles");
        return SHG_ERR_STATE;
    }
    h->batch.set_crystal(h->cfg);
    return SHG_OK;
}

int shg_get_temperature(shg_handle *h, float *T) {
    SHG_TRY(check_handle(h));
    if (!h->th || !h->th->has_result() || !T) {
        set_error("shg_get_temperature: needs a thermal handle after shg_run");
        return SHG_ERR_STATE;
    }
    return h->th->copy_temperature(T);
}

int shg_set_jacobi_rule(shg_handle *h, double rel_tol, int check_every, int max_sweeps) {
    SHG_TRY(check_handle(h));
    if (!h->th) {
        set_error("shg_set_jacobi_rule: needs a thermal handle");
        return SHG_ERR_STATE;
    }
    if (rel_tol > 0 && (check_every < 1 || max_sweeps < 1)) {
        set_error("shg_set_jacobi_rule: check_every and max_sweeps must be positive");
        return SHG_ERR_INVALID;
    }
    h->th->set_stop_rule(rel_tol, check_every, max_sweeps);
    return SHG_OK;
}

int shg_get_jacobi_residual(shg_handle *h, double *rel) {
    SHG_TRY(check_handle(h));
    if (!h->th || !rel) {
        set_error("shg_get_jacobi_residual: needs a thermal handle");
        return SHG_ERR_STATE;
    }
    *rel = h->th->last_residual();
    return SHG_OK;
}

int shg_get_jacobi_counts(shg_handle *h, int *counts) {
    SHG_TRY(check_handle(h));
    if (!h->th || !h->th->has_result() || !counts) {
        set_error("shg_get_jacobi_counts: needs a thermal handle after shg_run");
        return SHG_ERR_STATE;
    }
    h->th->counts(counts);
    return SHG_OK;
}

int shg_batch_create(const shg_config *crystal, const shg_instance *inst, int n, shg_batch **out) {
    if (!crystal || !inst || !out || n <= 0) {
        set_error("null argument or empty batch");
        return SHG_ERR_INVALID;
    }
    if (crystal->crystal != SHG_CRYSTAL_SPPLT && crystal->crystal != SHG_CRYSTAL_PPLN) {
        set_error("crystal must be SHG_CRYSTAL_SPPLT or SHG_CRYSTAL_PPLN");
        return SHG_ERR_INVALID;
    }
    *out = nullptr;
    std::vector<SolveParams> sp(n);
    for (int i = 0; i < n; ++i) {
        const shg_instance &s = inst[i];
        if (s.nx != s.ny) {
            set_error("batch solves must be square");
            return SHG_ERR_UNSUPPORTED;
        }
        sp[i] = SolveParams{s.nx, s.nz, s.lx, s.ly, s.power, s.waist, s.focal, s.temp, s.temp, s.temp};
    }
    auto *b = new shg_batch;
    b->cfg = *crystal;
    int rc = b->batch.create(*crystal, sp);
    if (rc) {
        delete b;
        return rc;
    }
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("stream creation failed");
        delete b;
        return SHG_ERR_CUDA;
    }
    *out = b;
    return SHG_OK;
}

int shg_batch_destroy(shg_batch *b) {
    delete b;
    return SHG_OK;
}

int shg_batch_run_async(shg_batch *b, void *stream) {
    shg::Phase phase("shg_batch_run_async");
    if (!b) {
        set_error("null batch");
        return SHG_ERR_INVALID;
    }
    SHG_TRY(b->batch.run_async(static_cast<cudaStream_t>(stream), true));
    b->ran = true;
    return SHG_OK;
}

int shg_batch_results(shg_batch *b, double *eta) {
    if (!b || !eta) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    if (!b->ran) {
        set_error("batch has not run");
        return SHG_ERR_STATE;
    }
    std::vector<double> acc;
    SHG_TRY(b->batch.copy_acc(acc));
    int bad = -1;
    for (int i = 0; i < b->batch.size(); ++i) {
        eta[i] = b->batch.eta_of(i, acc);
        if (bad < 0 && !std::isfinite(eta[i])) bad = i;
    }
    if (bad >= 0) {
        set_error("efficiency of solve " + std::to_string(bad) + " is not finite (every solve's value is stored)");
        return SHG_ERR_NONFINITE;
    }
    return SHG_OK;
}

int shg_batch_run(shg_batch *b, double *eta, float *sh_out_all) {
    shg::Phase phase("shg_batch_run");
    if (!b) {
        set_error("null batch");
        return SHG_ERR_INVALID;
    }
    SHG_TRY(b->batch.run_async(b->stream, true));
    b->ran = true;
    if (sh_out_all)
        SHG_CUDA(cudaMemcpyAsync(sh_out_all, b->batch.sout_all(), b->batch.total_points() * sizeof(float2),
                                 cudaMemcpyDeviceToHost, b->stream));
    SHG_CUDA(cudaStreamSynchronize(b->stream));
    if (eta)
        SHG_TRY(shg_batch_results(b, eta));
    else
        SHG_TRY(b->batch.check_run_errors());
    return SHG_OK;
}

int shg_batch_fields(shg_batch *b, float *pump_out_all, float *sh_out_all) {
    if (!b || !b->ran) {
        set_error("shg_batch_fields: batch has not run");
        return SHG_ERR_STATE;
    }
    SHG_CUDA(cudaStreamSynchronize(b->stream));
    SHG_TRY(b->batch.check_run_errors());
    const size_t bytes = b->batch.total_points() * sizeof(float2);
    if (pump_out_all) SHG_CUDA(cudaMemcpy(pump_out_all, b->batch.pout_all(), bytes, cudaMemcpyDeviceToHost));
    if (sh_out_all) SHG_CUDA(cudaMemcpy(sh_out_all, b->batch.sout_all(), bytes, cudaMemcpyDeviceToHost));
    return SHG_OK;
}

int shg_batch_set_instances(shg_batch *b, const shg_instance *inst, int n) {
    if (!b || !inst || n != b->batch.size()) {
        set_error("shg_batch_set_instances: null argument or solve count differs from the batch");
        return SHG_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i) {
        const shg_instance &s = inst[i];
        SHG_TRY(b->batch.set_params(i, SolveParams{s.nx, s.nz, s.lx, s.ly, s.power, s.waist, s.focal, s.temp,
                                                   s.temp, s.temp}));
    }
    return SHG_OK;
}

int shg_batch_field_offsets(shg_batch *b, long long *offsets) {
    if (!b || !offsets) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    for (int i = 0; i <= b->batch.size(); ++i)
        offsets[i] = (long long)(i < b->batch.size() ? b->batch.field_offset(i) : b->batch.total_points());
    return SHG_OK;
}

int shg_batch_profile(shg_batch *b, shg_kernel_stat *stats, int max_stats, int *n_stats) {
    if (!b || !stats || !n_stats || max_stats <= 0) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    Batch::Recorder rec;
    SHG_TRY(b->batch.profile(b->stream, rec));
    std::vector<std::string> order;
    std::map<std::string, shg_kernel_stat> acc;
    for (const auto &r : rec.recs) {
        float ms = 0.f;
        SHG_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        auto it = acc.find(r.name);
        if (it == acc.end()) {
            shg_kernel_stat z;
            std::memset(&z, 0, sizeof(z));
            std::snprintf(z.name, sizeof(z.name), "%s", r.name.c_str());
            it = acc.emplace(r.name, z).first;
            order.push_back(r.name);
        }
        it->second.launches += 1;
        it->second.ms += ms;
        it->second.bytes += r.bytes;
    }
    *n_stats = 0;
    for (const auto &nm : order) {
        if (*n_stats >= max_stats) break;
        stats[(*n_stats)++] = acc[nm];
    }
    b->ran = true;
    return SHG_OK;
}

int shg_batch_io_bytes(shg_batch *b, long long *h2d_per_run, long long *d2h_fields) {
    if (!b) {
        set_error("null batch");
        return SHG_ERR_INVALID;
    }
    if (h2d_per_run) *h2d_per_run = (long long)(b->batch.size() * (sizeof(shg_instance) + sizeof(InstDesc)));
    if (d2h_fields) *d2h_fields = (long long)(b->batch.total_points() * sizeof(float2));
    return SHG_OK;
}

int shg_batch_launch_count(shg_batch *b, int *launches) {
    if (!b || !launches) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    *launches = b->batch.launch_count();
    return SHG_OK;
}

int shg_batch_autotune(shg_batch *b, void *stream) {
    shg::Phase phase("shg_batch_autotune");
    if (!b) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SHG_TRY_INT(b->batch.tune(st));
    SHG_CUDA(cudaStreamSynchronize(st));
    return SHG_OK;
}

int shg_batch_timeline(shg_batch *b, double *start_end, int max_classes, int *n_classes, void *stream) {
    if (!b || !start_end || !n_classes) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    std::vector<double> se;
    SHG_TRY_INT(b->batch.timeline(static_cast<cudaStream_t>(stream), se));
    *n_classes = (int)se.size() / 2;
    for (int i = 0; i < (int)se.size() && i < 2 * max_classes; ++i) start_end[i] = se[i];
    return SHG_OK;
}

int shg_batch_set_schedule(shg_batch *b, int n, int resident, int cluster_size, int ctas_per_sm) {
    if (!b) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    return b->batch.set_schedule(n, resident, cluster_size, ctas_per_sm);
}

int shg_batch_set_schedule_split(shg_batch *b, int n, int cluster_size, int ctas_per_sm, int threads_per_line) {
    if (!b) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    return b->batch.set_schedule(n, 1, cluster_size, ctas_per_sm, threads_per_line);
}

int shg_batch_schedule(shg_batch *b, char *buf, int len) {
    if (!b || !buf || len <= 0) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    const std::string s = b->batch.schedule();
    std::snprintf(buf, (size_t)len, "%s", s.c_str());
    return (int)s.size() < len ? SHG_OK : SHG_ERR_INVALID;
}

int shg_check_status(int *enabled, int *site, long long *value) {
    if (!enabled || !site || !value) {
        set_error("null argument");
        return SHG_ERR_INVALID;
    }
    *enabled = kCheckBuild ? 1 : 0;
    *site = 0;
    *value = 0;
    if (!kCheckBuild) return SHG_OK;
    SHG_CUDA(cudaDeviceSynchronize());
    unsigned long long first = 0;
    for (auto take : {check_word_take_march, check_word_take_resident64, check_word_take_resident128,
                      check_word_take_resident256, check_word_take_cluster_pt, check_word_take_thermal,
                      check_word_take_heat_tma, check_word_take_adjoint}) {
        const unsigned long long w = take();
        if (w == ~0ull) {
            set_error("shg_check_status: status word unreadable");
            return SHG_ERR_CUDA;
        }
        if (w && !first) first = w;
    }
    if (first) {
        *site = (int)(first >> 48);
        long long v = (long long)(first & 0xffffffffffffull);
        if (v & (1ll << 47)) v -= 1ll << 48;  // sign of the 48-bit value
        *value = v;
    }
    return SHG_OK;
}

int shg_check_selftest(long long value) {
    if (!kCheckBuild) {
        set_error("shg_check_selftest: library built without SHG_CHECK");
        return SHG_ERR_UNSUPPORTED;
    }
    SHG_CUDA(launch_check_selftest(value));
    return SHG_OK;
}

int shg_dft2d_device(int n, int sign, const void *in, void *out, void *stream) {
    if (!line_length_supported(n) || (sign != 1 && sign != -1) || !in || !out) {
        set_error("shg_dft2d_device: unsupported size or bad argument");
        return SHG_ERR_INVALID;
    }
    int dev = 0;
    SHG_CUDA(cudaGetDevice(&dev));
    SHG_TRY(ensure_twiddles(dev));
    SHG_CUDA(launch_dft2d(n, sign, static_cast<const float2 *>(in), static_cast<float2 *>(out),
                          static_cast<cudaStream_t>(stream)));
    return SHG_OK;
}

}  // extern "C"
