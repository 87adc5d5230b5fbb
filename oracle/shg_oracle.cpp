// ORACLE — test infrastructure only (see shg_oracle.h). Restates the reference's
// algorithm; every function names the reference lines it follows. The f32 path keeps
// the reference's float operation order and its implicit double sub-expressions; the f64
// path is the same method in double.
#include "shg_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

#include "dft_ref.h"

namespace {

using D = double;

template <class R>
struct cx {
    R re, im;
};

// Operators.h:13-101 — the reference's own complex overloads (naive forms).
template <class R> inline cx<R> add(cx<R> a, cx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <class R> inline cx<R> sub(cx<R> a, cx<R> b) { return {a.re - b.re, a.im - b.im}; }
template <class R> inline cx<R> neg(cx<R> a) { return {-a.re, -a.im}; }
template <class R> inline cx<R> mul(cx<R> a, cx<R> b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class R> inline cx<R> mul_rc(R a, cx<R> b) { return {a * b.re, a * b.im}; }
template <class R> inline cx<R> div_cr(cx<R> b, R a) { return {b.re / a, b.im / a}; }
template <class R> inline cx<R> div_rc(R a, cx<R> b) {
    R den = b.re * b.re + b.im * b.im;
    return {(+a * b.re) / den, (-a * b.im) / den};
}
template <class R> inline cx<R> conj(cx<R> a) { return {+a.re, -a.im}; }
template <class R> inline R abs2(cx<R> a) { return a.re * a.re + a.im * a.im; }

inline float f_cos(float a) { return cosf(a); }
inline float f_sin(float a) { return sinf(a); }
inline float f_exp(float a) { return expf(a); }
inline float f_sqrt(float a) { return sqrtf(a); }
inline float f_tan(float a) { return tanf(a); }
inline double f_cos(double a) { return std::cos(a); }
inline double f_sin(double a) { return std::sin(a); }
inline double f_exp(double a) { return std::exp(a); }
inline double f_sqrt(double a) { return std::sqrt(a); }
inline double f_tan(double a) { return std::tan(a); }

// Operators.h:105-117
template <class R> inline cx<R> cexp_real(R a) { return {f_cos(a), f_sin(a)}; }
template <class R> inline cx<R> cexp_cpx(cx<R> a) {
    return {f_exp(a.re) * f_cos(a.im), f_exp(a.re) * f_sin(a.im)};
}

// Crystal.h:116-132. Float arguments and coefficients; pow and sqrt in double; the
// result is rounded to R. (b and c are rounded to R on assignment, (B+b) and (C+c) are
// R sums.)
template <class R>
R sellmeier(R L, R T) {
    const R A = (R)4.502483, B = (R)0.007294, C = (R)0.185087, Dd = (R)-0.02357;
    const R E = (R)0.073423, F = (R)0.199595, G = (R)0.001, H = (R)7.99724;
    const D tk = (D)T + 273.15;
    const R b = (R)(3.483933e-8 * (tk * tk));
    const R c = (R)(1.607839e-8 * (tk * tk));
    const D L2 = (D)L * (D)L;
    const R Cc = C + c;
    const R Bb = B + b;
    const D n2 = (D)A + (D)Bb / (L2 - (D)Cc * (D)Cc) + (D)E / (L2 - (D)F * (D)F) +
                 (D)G / (L2 - (D)H * (D)H) + (D)Dd * L2;
    return (R)std::sqrt(n2);
}

// PPLN (congruent LiNbO3) extraordinary index, the fit of D. H. Jundt, Opt. Lett. 22,
// 1553-1555 (1997): n^2 = a1 + b1 f + (a2 + b2 f)/(L^2 - (a3 + b3 f)^2) + (a4 + b4 f)/(L^2 - a5^2)
// - a6 L^2, f = (T - 24.5)(T + 570.82); double, rounded to R. Not part of the reference's code
// (its README names an MgO:PPLN crystal): a restatement of the published fit, evaluated in
// the same operation order as the device code.
template <class R>
R lithium_niobate(R L, R T) {
    const D a1 = 5.35583, a2 = 0.100473, a3 = 0.20692, a4 = 100.0, a5 = 11.34927, a6 = 1.5334e-2;
    const D b1 = 4.629e-7, b2 = 3.862e-8, b3 = -0.89e-8, b4 = 2.657e-5;
    const D t = (D)T, L2 = (D)L * (D)L;
    const D f = (t - 24.5) * (t + 570.82);
    const D c3 = a3 + b3 * f;
    const D n2 = a1 + b1 * f + (a2 + b2 * f) / (L2 - c3 * c3) + (a4 + b4 * f) / (L2 - a5 * a5) - a6 * L2;
    return (R)std::sqrt(n2);
}

template <class R>
R crystal_n(int crystal, R L, R T) {
    return crystal == 1 ? lithium_niobate<R>(L, T) : sellmeier<R>(L, T);
}

// Crystal.h:80-82 and the per-configuration constants of Crystal.h:26-53.
template <class R>
struct Model {
    int NX, NY, NZ, crystal;
    size_t NXY, TSIZE;
    R PI, Cl, EPS0, lp, ls, LX, LY, LZ, dx, dy, dz, deff, dQ, Lambda, alpha_crp, alpha_crs, beta_crs,
        rhop, rhos, thermal_cond, heat_trf_coeff;

    explicit Model(const oracle_cfg &c) {
        NX = c.nx;
        NY = c.ny;
        NZ = c.nz;
        crystal = c.crystal;
        NXY = (size_t)NX * NY;
        TSIZE = NXY * (size_t)NZ;
        PI = (R)3.14159265358979323846;
        Cl = (R)(299792458 * 1E6 / 1E12);
        EPS0 = (R)(8.8541878128E-12 * 1E12 / 1E6);
        lp = (R)c.lp;
        ls = (R)(0.5 * (D)lp);
        LX = (R)c.lx;
        LY = (R)c.ly;
        LZ = (R)c.lz;
        dx = LX / (R)(unsigned)(NX - 1);
        dy = LY / (R)(unsigned)(NY - 1);
        dz = LZ / (R)(unsigned)(NZ - 1);
        deff = (R)c.deff;
        dQ = (R)((2.0 / (D)PI) * (D)deff);
        Lambda = (R)c.lambda_qpm;
        alpha_crp = (R)c.alpha_p;
        alpha_crs = (R)c.alpha_s;
        beta_crs = (R)c.beta_s;
        rhop = (R)c.rho_p;
        rhos = (R)c.rho_s;
        thermal_cond = (R)c.kth;
        heat_trf_coeff = (R)c.htc;
    }
    size_t idx(int x, int y, int z) const { return (size_t)z * NXY + (size_t)y * NX + x; }
    R n(R L, R T) const { return crystal_n<R>(crystal, L, T); }
};

template <class R>
using cvec = std::vector<cx<R>>;

// Efields.h:74-104 (setPump), with Temp = T at the grid centre of slice 0.
template <class R>
void set_pump(const Model<R> &m, R Power, R focalpoint, R waistX, R Temp, cx<R> *Pump) {
    const R PI = (R)3.14159265358979323846;
    const cx<R> Im{(R)0, (R)1};
    const R uX = (R)(0.5 * m.NX);
    const R uY = (R)(0.5 * m.NY);
    const R waistY = waistX;
    const R wX2 = waistX * waistX;
    const R wY2 = waistY * waistY;
    (void)wY2;
    const R zRX = PI * m.n(m.lp, Temp) * wX2 / m.lp;
    const R Ap0 = f_sqrt((R)4 * Power / (m.EPS0 * m.Cl * PI * m.n(m.lp, Temp) * wX2));
    const R etaX = focalpoint / zRX;
    // (1 - Im*etaX): Operators.h:67 then :39
    const cx<R> ImEta = {etaX * Im.re, etaX * Im.im};
    const cx<R> MX = {(R)1 - ImEta.re, -ImEta.im};
    const cx<R> amp = div_rc<R>(Ap0, MX);
    const cx<R> wM = mul_rc<R>(wX2, MX);
    for (int ix = 0; ix < m.NX; ++ix) {
        for (int iy = 0; iy < m.NY; ++iy) {
            const R ax = ((R)(unsigned)ix - uX) * m.dx;
            const R ay = ((R)(unsigned)iy - uY) * m.dy;
            const R num = -(ax * ax) - (ay * ay);
            Pump[m.idx(ix, iy, 0)] = mul(amp, cexp_cpx(div_rc<R>(num, wM)));
        }
    }
}

// Efields.h:32-71 (fftShift2DV then fftShift2DH, including the odd-size behaviour).
template <class R>
void fft_shift_2d(const Model<R> &m, cx<R> *F) {
    cvec<R> aux(F, F + m.NXY);
    const int r = (int)std::floor((R)m.NY / 2);
    for (int iy = 0; iy < r; ++iy)
        for (int ix = 0; ix < m.NX; ++ix) {
            F[m.idx(ix, iy + r, 0)] = aux[m.idx(ix, iy, 0)];
            F[m.idx(ix, iy, 0)] = aux[m.idx(ix, iy + r, 0)];
        }
    aux.assign(F, F + m.NXY);
    const int c = (int)std::floor((R)m.NX / 2);
    for (int iy = 0; iy < m.NY; ++iy)
        for (int ix = 0; ix < c; ++ix) {
            F[m.idx(ix + c, iy, 0)] = aux[m.idx(ix, iy, 0)];
            F[m.idx(ix, iy, 0)] = aux[m.idx(ix + c, iy, 0)];
        }
}

// Efields.h:107-126 (beamPropagator) followed by the shifts of Efields.h:186-192.
template <class R>
void propagators(const Model<R> &m, R Temp, cx<R> *hp, cx<R> *hs) {
    const R PI = (R)3.14159265358979323846;
    const R kp = (R)2 * PI * m.n(m.lp, Temp) / m.lp;
    const R ks = (R)2 * PI * m.n(m.ls, Temp) / m.ls;
    const R dfX = (R)1 / m.dx / (R)(unsigned)m.NX;
    const R dfY = (R)1 / m.dy / (R)(unsigned)m.NY;
    const R uX = (R)(0.5 * m.NX);
    const R uY = (R)(0.5 * m.NY);
    const R pi2 = PI * PI;
    const R tp = f_tan(m.rhop), ts = f_tan(m.rhos);
    for (int iy = 0; iy < m.NY; ++iy)
        for (int ix = 0; ix < m.NX; ++ix) {
            const R tx = (R)(unsigned)ix - uX;
            const R ty = (R)(unsigned)iy - uY;
            const R q = dfX * dfX * (tx * tx) + dfY * dfY * (ty * ty);
            const R ap = -m.dz * ((R)2 * pi2 / kp * q + (R)2 * PI * dfX * tp * tx);
            const R as = -m.dz * ((R)2 * pi2 / ks * q + (R)2 * PI * dfX * ts * tx);
            hp[m.idx(ix, iy, 0)] = cexp_real(ap);
            hs[m.idx(ix, iy, 0)] = cexp_real(as);
        }
    fft_shift_2d(m, hp);
    fft_shift_2d(m, hs);
}

// PhaseMatching.h:57-70 (one element of the constant table).
template <class R>
R dk_constant(const Model<R> &m, R Temp) {
    const R PI = m.PI;
    return (R)2 * PI * ((R)2 * m.n(m.lp, Temp) / m.lp - m.n(m.ls, Temp) / m.ls + (R)1 / (m.Lambda));
}

// Solver.h:156-190 + Efields.h:15-30 (FFTW_BACKWARD, propagator product, FFTW_FORWARD,
// scale by 1/(NX*NY) as a division).
template <class R>
void diffraction(const Model<R> &m, const cx<R> *hp, const cx<R> *hs, cx<R> *P, cx<R> *S,
                 cvec<R> &work) {
    work.resize(m.NXY);
    const R size = (R)(unsigned)(m.NX * m.NY);
    for (int f = 0; f < 2; ++f) {
        cx<R> *A = f == 0 ? P : S;
        const cx<R> *H = f == 0 ? hp : hs;
        dftref::dft2d<R>(reinterpret_cast<R *>(A), reinterpret_cast<R *>(work.data()), m.NX, m.NY, +1);
        for (size_t i = 0; i < m.NXY; ++i) work[i] = mul(H[i], work[i]);
        dftref::dft2d<R>(reinterpret_cast<R *>(work.data()), reinterpret_cast<R *>(A), m.NX, m.NY, -1);
        for (size_t i = 0; i < m.NXY; ++i) A[i] = div_cr<R>(A[i], size);
    }
}

// Solver.h:65-83 (dAdz without THERMAL). The indices are evaluated per pixel, as there.
template <class R>
void dadz_plain(const Model<R> &m, cx<R> *dP, cx<R> *dS, const cx<R> *P, const cx<R> *S, R DK,
                R Temp, R z) {
    const R PI = (R)3.14159265358979323846;
    const cx<R> Im{(R)0, (R)1};
    for (int iy = 0; iy < m.NY; ++iy)
        for (int ix = 0; ix < m.NX; ++ix) {
            const size_t i = m.idx(ix, iy, 0);
            const R np = m.n(m.lp, Temp), ns = m.n(m.ls, Temp);
            // Im*1.0*PI*dQ/(n*lp) * Signal * CpxConj(Pump) * CpxExp(-Im*z*DK) - 0.5*alpha*Pump
            cx<R> t = mul_rc<R>((R)1.0, Im);
            t = mul_rc<R>(PI, t);
            t = mul_rc<R>(m.dQ, t);
            t = div_cr<R>(t, np * m.lp);
            t = mul(t, S[i]);
            t = mul(t, conj(P[i]));
            const cx<R> arg = mul_rc<R>(DK, mul_rc<R>(z, neg(Im)));
            t = mul(t, cexp_cpx(arg));
            dP[i] = sub(t, mul_rc<R>((R)(0.5 * (D)m.alpha_crp), P[i]));
            // Im*0.5*PI*dQ/(n*ls) * Pump * Pump * CpxExp(+z*DK)
            //   - 0.5*(alpha_crs + beta_crs*0.5*C*EPS0*n*CpxAbs2(Signal)) * Signal
            cx<R> u = mul_rc<R>((R)0.5, Im);
            u = mul_rc<R>(PI, u);
            u = mul_rc<R>(m.dQ, u);
            u = div_cr<R>(u, ns * m.ls);
            u = mul(u, P[i]);
            u = mul(u, P[i]);
            u = mul(u, cexp_real<R>(z * DK));
            const D tpa = 0.5 * ((D)m.alpha_crs + (D)m.beta_crs * 0.5 * (D)m.Cl * (D)m.EPS0 * (D)ns *
                                                      (D)abs2(S[i]));
            dS[i] = sub(u, mul_rc<R>((R)tpa, S[i]));
        }
}

// Solver.h:44-63 (dAdz with THERMAL): n from T(x,y,s); phase DKint*(dz*inc+(s+1)*dz)/(s+1)
// evaluated in double (the literal 1.0 promotes it) and passed to CpxExp(real).
template <class R>
void dadz_thermal(const Model<R> &m, cx<R> *dP, cx<R> *dS, const cx<R> *P, const cx<R> *S,
                  const R *T, const R *DKint, R increment, int s) {
    const R PI = (R)3.14159265358979323846;
    const cx<R> Im{(R)0, (R)1};
    for (int iy = 0; iy < m.NY; ++iy)
        for (int ix = 0; ix < m.NX; ++ix) {
            const size_t i = m.idx(ix, iy, 0);
            const R Tl = T[m.idx(ix, iy, s)];
            const D sp1 = (D)(unsigned)s + 1.0;
            const D ph = (D)DKint[i] * ((D)(m.dz * increment) + sp1 * (D)m.dz) / sp1;
            cx<R> t = mul_rc<R>((R)1.0, Im);
            t = mul_rc<R>(PI, t);
            t = mul_rc<R>(m.dQ, t);
            t = div_cr<R>(t, m.n(m.lp, Tl) * m.lp);
            t = mul(t, S[i]);
            t = mul(t, conj(P[i]));
            t = mul(t, cexp_real<R>((R)(-ph)));
            dP[i] = sub(t, mul_rc<R>((R)(0.5 * (D)m.alpha_crp), P[i]));
            cx<R> u = mul_rc<R>((R)0.5, Im);
            u = mul_rc<R>(PI, u);
            u = mul_rc<R>(m.dQ, u);
            u = div_cr<R>(u, m.n(m.ls, Tl) * m.ls);
            u = mul(u, P[i]);
            u = mul(u, P[i]);
            u = mul(u, cexp_real<R>((R)(+ph)));
            const D tpa = 0.5 * ((D)m.alpha_crs + (D)m.beta_crs * 0.5 * (D)m.EPS0 * (D)m.Cl *
                                                      (D)m.n(m.ls, Tl) * (D)abs2(S[i]));
            dS[i] = sub(u, mul_rc<R>((R)tpa, S[i]));
        }
}

template <class R>
struct RK4Work {
    cvec<R> k1p, k2p, k3p, k4p, k1s, k2s, k3s, k4s, auxp, auxs, diff;
    std::vector<R> DKint;
    explicit RK4Work(size_t n)
        : k1p(n), k2p(n), k3p(n), k4p(n), k1s(n), k2s(n), k3s(n), k4s(n), auxp(n), auxs(n), DKint(n) {}
};

// Solver.h:103-117
template <class R>
void lin_comb(const Model<R> &m, cx<R> *ap, cx<R> *as, const cx<R> *P, const cx<R> *S, const cx<R> *kp,
              const cx<R> *ks, R c) {
    for (size_t i = 0; i < m.NXY; ++i) {
        ap[i] = add(P[i], mul_rc<R>(c, kp[i]));
        as[i] = add(S[i], mul_rc<R>(c, ks[i]));
    }
}

// Solver.h:86-100: A + (k1 + 2k2 + 2k3 + k4) * dz / 6
template <class R>
void sum_rk4(const Model<R> &m, cx<R> *P, cx<R> *S, RK4Work<R> &w) {
    for (size_t i = 0; i < m.NXY; ++i) {
        cx<R> sp = add(add(add(w.k1p[i], mul_rc<R>((R)2, w.k2p[i])), mul_rc<R>((R)2, w.k3p[i])), w.k4p[i]);
        P[i] = add(P[i], div_cr<R>(mul_rc<R>(m.dz, sp), (R)6));
        cx<R> ss = add(add(add(w.k1s[i], mul_rc<R>((R)2, w.k2s[i])), mul_rc<R>((R)2, w.k3s[i])), w.k4s[i]);
        S[i] = add(S[i], div_cr<R>(mul_rc<R>(m.dz, ss), (R)6));
    }
}

// Solver.h:193-233 (solverRK4), both branches. The plain branch ignores `increment`.
template <class R>
void solver_rk4(const Model<R> &m, cx<R> *P, cx<R> *S, RK4Work<R> &w, bool thermal, R DK, R Temp,
                R z, const R *T, const R *DK3, int slice) {
    if (thermal) {
        // PhaseMatching.h:12-38: DKint = sum_{z'=0..s} DK(z'), from zero.
        for (size_t i = 0; i < m.NXY; ++i) w.DKint[i] = (R)0;
        for (int iz = 0; iz <= slice; ++iz)
            for (size_t i = 0; i < m.NXY; ++i) w.DKint[i] += DK3[(size_t)iz * m.NXY + i];
        const R inc[4] = {(R)(0.5 * 0.0), (R)(0.5 * 0.5), (R)(0.5 * 0.5), (R)(0.5 * 1.0)};
        dadz_thermal(m, w.k1p.data(), w.k1s.data(), P, S, T, w.DKint.data(), inc[0], slice);
        lin_comb(m, w.auxp.data(), w.auxs.data(), P, S, w.k1p.data(), w.k1s.data(), (R)0.5);
        dadz_thermal(m, w.k2p.data(), w.k2s.data(), w.auxp.data(), w.auxs.data(), T, w.DKint.data(), inc[1], slice);
        lin_comb(m, w.auxp.data(), w.auxs.data(), P, S, w.k2p.data(), w.k2s.data(), (R)0.5);
        dadz_thermal(m, w.k3p.data(), w.k3s.data(), w.auxp.data(), w.auxs.data(), T, w.DKint.data(), inc[2], slice);
        lin_comb(m, w.auxp.data(), w.auxs.data(), P, S, w.k3p.data(), w.k3s.data(), (R)1.0);
        dadz_thermal(m, w.k4p.data(), w.k4s.data(), w.auxp.data(), w.auxs.data(), T, w.DKint.data(), inc[3], slice);
    } else {
        dadz_plain(m, w.k1p.data(), w.k1s.data(), P, S, DK, Temp, z);
        lin_comb(m, w.auxp.data(), w.auxs.data(), P, S, w.k1p.data(), w.k1s.data(), (R)0.5);
        dadz_plain(m, w.k2p.data(), w.k2s.data(), w.auxp.data(), w.auxs.data(), DK, Temp, z);
        lin_comb(m, w.auxp.data(), w.auxs.data(), P, S, w.k2p.data(), w.k2s.data(), (R)0.5);
        dadz_plain(m, w.k3p.data(), w.k3s.data(), w.auxp.data(), w.auxs.data(), DK, Temp, z);
        lin_comb(m, w.auxp.data(), w.auxs.data(), P, S, w.k3p.data(), w.k3s.data(), (R)1.0);
        dadz_plain(m, w.k4p.data(), w.k4s.data(), w.auxp.data(), w.auxs.data(), DK, Temp, z);
    }
    sum_rk4(m, P, S, w);
}

// Tfield.h:277-290 (setQ): Q(x,y,s) from the fields after step s.
template <class R>
void set_q(const Model<R> &m, R *Q, const R *T, const cx<R> *P, const cx<R> *S, int s) {
    for (int iy = 0; iy < m.NY; ++iy)
        for (int ix = 0; ix < m.NX; ++ix) {
            const size_t i2 = m.idx(ix, iy, 0), i3 = m.idx(ix, iy, s);
            const R Tl = T[i3];
            const D t1 = (D)m.alpha_crp * 0.5 * (D)m.Cl * (D)m.EPS0 * (D)m.n(m.lp, Tl) * (D)abs2(P[i2]);
            const D t2 = (D)m.alpha_crs * 0.5 * (D)m.Cl * (D)m.EPS0 * (D)m.n(m.ls, Tl) * (D)abs2(S[i2]);
            const R in3 = (R)(0.5 * (D)m.Cl * (D)m.EPS0 * (D)m.n(m.ls, Tl) * (D)abs2(S[i2]));
            const R t3 = m.beta_crs * (in3 * in3);
            Q[i3] = (R)(t1 + t2 + (D)t3);
        }
}

// Solver.h:245-276 (CWES) with fields in memory; Q updates when thermal.
template <class R>
void cwes(const Model<R> &m, cx<R> *P, cx<R> *S, const cx<R> *hp, const cx<R> *hs, bool thermal,
          R DK, R Temp, const R *T, const R *DK3, R *Q, cx<R> *out_p, cx<R> *out_s) {
    RK4Work<R> w(m.NXY);
    R z = (R)0.0;
    for (int s = 0; s < m.NZ; ++s) {
        if (s == m.NZ - 1) {
            if (out_p) std::memcpy(out_p, P, m.NXY * sizeof(cx<R>));
            if (out_s) std::memcpy(out_s, S, m.NXY * sizeof(cx<R>));
        }
        // Solver.h:236-242 (SSFM): RK4, diffraction, RK4 at the same z.
        solver_rk4(m, P, S, w, thermal, DK, Temp, z, T, DK3, s);
        diffraction(m, hp, hs, P, S, w.diff);
        solver_rk4(m, P, S, w, thermal, DK, Temp, z, T, DK3, s);
        if (thermal) set_q(m, Q, T, P, S, s);
        z += m.dz;
    }
}

// Efields.h:129-144 with a fixed seed (same engine, distribution and draw order).
void noise_f32(size_t n, unsigned seed, cx<float> *A) {
    std::default_random_engine generator(seed);
    std::normal_distribution<float> distribution(0.0, 1.0e-20);
    for (size_t i = 0; i < n; ++i) {
        float a1 = distribution(generator);
        float a2 = distribution(generator);
        A[i] = {a1, a2};
    }
}

// Tfield.h:31-110
void init_temperature(const Model<float> &m, float *T, float Temp, float T1, float T2, int bc) {
    for (size_t i = 0; i < m.TSIZE; ++i) T[i] = Temp;
    const float nz = (float)m.NZ;
    if (bc == 0) {
        for (int iz = 0; iz < m.NZ; ++iz)
            for (int ix = 0; ix < m.NX; ++ix) {
                if (iz < nz / 2.0) T[m.idx(ix, 0, iz)] = T1;
                if (iz >= nz / 2.0) T[m.idx(ix, 0, iz)] = T2;
            }
    } else {
        for (int iz = 0; iz < m.NZ; ++iz)
            for (int iy = 0; iy < m.NY; ++iy)
                for (int ix = 0; ix < m.NX; ++ix) {
                    const bool lateral = iy == 0 || iy == m.NY - 1 || ix == 0 || ix == m.NX - 1;
                    if (lateral) T[m.idx(ix, iy, iz)] = (iz < nz / 2.0) ? T1 : T2;
                }
    }
}

// Coefficients of Tfield.h:118-125 (float, except the 0.5*(Bi+Bi) terms that the double
// literal promotes before the reciprocal is rounded to float).
struct HeatCoef {
    float Bix, Biy, Biz, ax, ay, az, bx, by, bz, av, bv, cv, V, ah, bh, ch, H, ad, bd, cd, Dd, AV, BV, CV, BiD,
        GV, L2, dx2, dy2, dz2, kth;
    explicit HeatCoef(const Model<float> &m) {
        const float dx = m.dx, dy = m.dy, dz = m.dz, k = m.thermal_cond, h = m.heat_trf_coeff;
        Bix = h * dx / k; Biy = h * dy / k; Biz = h * dz / k;
        ax = dx * dx / (2 * dy * dy); ay = dy * dy / (2 * dx * dx); az = dz * dz / (2 * dx * dx);
        bx = dx * dx / (2 * dz * dz); by = dy * dy / (2 * dz * dz); bz = dz * dz / (2 * dy * dy);
        av = dz / (2 * dx); bv = dx / (2 * dz); cv = dx * dz / (4 * dy * dy);
        V = (float)(1 / ((D)(av + bv + 2 * cv) + 0.5 * (D)(Bix + Biz)));
        ah = dz / (2 * dy); bh = dy / (2 * dz); ch = dy * dz / (4 * dx * dx);
        H = (float)(1 / ((D)(ah + bh + 2 * ch) + 0.5 * (D)(Biy + Biz)));
        ad = dx / (2 * dy); bd = dy / (2 * dx); cd = dx * dy / (4 * dz * dz);
        Dd = (float)(1 / ((D)(ad + bd + 2 * cd) + 0.5 * (D)(Bix + Biy)));
        AV = dy * dz / dx; BV = dx * dz / dy; CV = dx * dy / dz;
        BiD = Bix * dy + Biy * dz + Biz * dx;
        GV = 1 / (AV + BV + CV + BiD);
        L2 = 1 / (2 / (dx * dx) + 2 / (dy * dy) + 2 / (dz * dz));
        dx2 = dx * dx; dy2 = dy * dy; dz2 = dz * dz; kth = k;
    }
};

// Host threads of the heat sweep (oracle_set_threads). Every voxel of a sweep depends only
// on the previous sweep's field, so splitting the z range over threads changes no result.
static int g_heat_threads = 1;

// One sweep of Tfield.h:113-221 (bc 0) or Tfield.h:224-258 (bc 1), planes [z0, z1): Tf from
// Ti. Voxels that the reference never writes keep Tf's current value.
void heat_sweep_planes(const Model<float> &m, const HeatCoef &c, float *Tf, const float *Ti, float T_inf,
                       const float *Q, int bc, int z0, int z1) {
    const int NX = m.NX, NY = m.NY, NZ = m.NZ;
    auto I = [&](int x, int y, int z) { return m.idx(x, y, z); };
    for (int z = z0; z < z1; ++z)
        for (int y = 0; y < NY; ++y)
            for (int x = 0; x < NX; ++x) {
                const bool xi = x > 0 && x < NX - 1, yi = y > 0 && y < NY - 1, zi = z > 0 && z < NZ - 1;
                float *o = &Tf[I(x, y, z)];
                if (xi && yi && zi) {
                    *o = c.L2 * ((Ti[I(x + 1, y, z)] + Ti[I(x - 1, y, z)]) / c.dx2 +
                                 (Ti[I(x, y + 1, z)] + Ti[I(x, y - 1, z)]) / c.dy2 +
                                 (Ti[I(x, y, z + 1)] + Ti[I(x, y, z - 1)]) / c.dz2 + Q[I(x, y, z)] / c.kth);
                    continue;
                }
                if (xi && yi && (z == 0 || z == NZ - 1)) {  // back / front faces
                    const int zn = z == 0 ? z + 1 : z - 1;
                    *o = (Ti[I(x, y, zn)] + c.az * (Ti[I(x + 1, y, z)] + Ti[I(x - 1, y, z)]) +
                          c.bz * (Ti[I(x, y + 1, z)] + Ti[I(x, y - 1, z)]) + c.Biz * T_inf) /
                         (1 + 2 * c.az + 2 * c.bz + c.Biz);
                    continue;
                }
                if (bc != 0) continue;  // oven surrounded: lateral faces are fixed
                if ((x == 0 || x == NX - 1) && yi && zi) {  // left / right faces
                    const int xn = x == 0 ? x + 1 : x - 1;
                    *o = (Ti[I(xn, y, z)] + c.ax * (Ti[I(x, y + 1, z)] + Ti[I(x, y - 1, z)]) +
                          c.bx * (Ti[I(x, y, z + 1)] + Ti[I(x, y, z - 1)]) + c.Bix * T_inf) /
                         (1 + 2 * c.ax + 2 * c.bx + c.Bix);
                } else if (xi && y == NY - 1 && zi) {  // top face
                    *o = (Ti[I(x, y - 1, z)] + c.ay * (Ti[I(x + 1, y, z)] + Ti[I(x - 1, y, z)]) +
                          c.by * (Ti[I(x, y, z + 1)] + Ti[I(x, y, z - 1)]) + c.Biy * T_inf) /
                         (1 + 2 * c.ay + 2 * c.by + c.Biy);
                } else if ((x == 0 || x == NX - 1) && yi && (z == 0 || z == NZ - 1)) {  // vertical sides
                    const int xn = x == 0 ? x + 1 : x - 1, zn = z == 0 ? z + 1 : z - 1;
                    const float s = c.av * Ti[I(xn, y, z)] + c.bv * Ti[I(x, y, zn)] +
                                    c.cv * (Ti[I(x, y + 1, z)] + Ti[I(x, y - 1, z)]);
                    *o = (float)(((D)s + 0.5 * (D)T_inf * (D)(c.Bix + c.Biz)) * (D)c.V);
                } else if (y == NY - 1 && xi && (z == 0 || z == NZ - 1)) {  // horizontal sides
                    const int zn = z == 0 ? z + 1 : z - 1;
                    const float s = c.ah * Ti[I(x, y - 1, z)] + c.bh * Ti[I(x, y, zn)] +
                                    c.ch * (Ti[I(x - 1, y, z)] + Ti[I(x + 1, y, z)]);
                    *o = (float)(((D)s + 0.5 * (D)T_inf * (D)(c.Biy + c.Biz)) * (D)c.H);
                } else if ((x == 0 || x == NX - 1) && y == NY - 1 && zi) {  // depth sides
                    const int xn = x == 0 ? x + 1 : x - 1;
                    const float s = c.ad * Ti[I(x, y - 1, z)] + c.bd * Ti[I(xn, y, z)] +
                                    c.cd * (Ti[I(x, y, z + 1)] + Ti[I(x, y, z - 1)]);
                    *o = (float)(((D)s + 0.5 * (D)T_inf * (D)(c.Bix + c.Biy)) * (D)c.Dd);
                } else if ((x == 0 || x == NX - 1) && y == NY - 1 && (z == 0 || z == NZ - 1)) {  // vertices
                    const int xn = x == 0 ? x + 1 : x - 1, zn = z == 0 ? z + 1 : z - 1;
                    *o = (c.AV * Ti[I(xn, y, z)] + c.BV * Ti[I(x, y - 1, z)] + c.CV * Ti[I(x, y, zn)] +
                          T_inf * c.BiD) * c.GV;
                }
            }
}

void heat_sweep(const Model<float> &m, const HeatCoef &c, float *Tf, const float *Ti, float T_inf,
                const float *Q, int bc) {
    const int NZ = m.NZ, nt = std::max(1, std::min(g_heat_threads, NZ));
    if (nt == 1) {
        heat_sweep_planes(m, c, Tf, Ti, T_inf, Q, bc, 0, NZ);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back(heat_sweep_planes, std::cref(m), std::cref(c), Tf, Ti, T_inf, Q, bc, NZ * t / nt,
                          NZ * (t + 1) / nt);
    for (auto &th : pool) th.join();
}

// Tfield.h:13-28
float reduced_sum(const Model<float> &m, const float *Tf, const float *Ti) {
    float sum = 0.0;
    for (size_t i = 0; i < m.TSIZE; ++i) {
        const float d = Tf[i] - Ti[i];
        sum += d * d;
    }
    return sum / (float)(unsigned)m.TSIZE;
}

// PhaseMatching.h:41-54
template <class R>
void dk_thermal(const Model<R> &m, const R *T, R *DK) {
    const R PI = m.PI;
    for (size_t i = 0; i < m.TSIZE; ++i)
        DK[i] = (R)2 * PI * ((R)2 * m.n(m.lp, T[i]) / m.lp - m.n(m.ls, T[i]) / m.ls + (R)1 / (m.Lambda));
}

template <class R>
double power_of(const Model<R> &m, const cx<R> *A, R nidx) {
    double s = 0.0;
    for (size_t i = 0; i < m.NXY; ++i) s += (double)A[i].re * A[i].re + (double)A[i].im * A[i].im;
    return 0.5 * (double)m.EPS0 * (double)m.Cl * (double)nidx * s * (double)m.dx * (double)m.dy;
}

template <class R>
cx<R> *as_cx(R *p) { return reinterpret_cast<cx<R> *>(p); }
template <class R>
const cx<R> *as_cx(const R *p) { return reinterpret_cast<const cx<R> *>(p); }

// Solver.h:245-276 (THERMAL) from given fields with the temperature field held fixed;
// DK3 == nullptr: delta-k(T) in R, else the given table (to pin the float delta-k).
template <class R>
void cwes_thermal_impl(const oracle_cfg *c, const R *T, const R *DK3, const R *pump, const R *sh, R tc,
                       R *out_pump, R *out_sh) {
    Model<R> m(*c);
    cvec<R> P(as_cx(pump), as_cx(pump) + m.NXY), S(as_cx(sh), as_cx(sh) + m.NXY);
    cvec<R> hp(m.NXY), hs(m.NXY);
    propagators<R>(m, tc, hp.data(), hs.data());
    std::vector<R> dk(m.TSIZE), Q(m.TSIZE);
    if (DK3)
        std::copy(DK3, DK3 + m.TSIZE, dk.begin());
    else
        dk_thermal<R>(m, T, dk.data());
    cwes<R>(m, P.data(), S.data(), hp.data(), hs.data(), true, (R)0, tc, T, dk.data(), Q.data(),
            out_pump ? as_cx(out_pump) : nullptr, out_sh ? as_cx(out_sh) : nullptr);
}

template <class R>
void cwes_plain_impl(const oracle_cfg *c, const R *pump, const R *sh, R temp, R dk, R *out_pump,
                            R *out_sh, R *end_pump, R *end_sh) {
    Model<R> m(*c);
    cvec<R> P(as_cx(pump), as_cx(pump) + m.NXY), S(as_cx(sh), as_cx(sh) + m.NXY);
    cvec<R> hp(m.NXY), hs(m.NXY);
    propagators<R>(m, temp, hp.data(), hs.data());
    if (std::isnan((double)dk)) dk = dk_constant<R>(m, temp);
    cwes<R>(m, P.data(), S.data(), hp.data(), hs.data(), false, dk, temp, nullptr, nullptr, nullptr,
            out_pump ? as_cx(out_pump) : nullptr, out_sh ? as_cx(out_sh) : nullptr);
    if (end_pump) std::memcpy(end_pump, P.data(), m.NXY * sizeof(cx<R>));
    if (end_sh) std::memcpy(end_sh, S.data(), m.NXY * sizeof(cx<R>));
}

}  // namespace

extern "C" {

float oracle_n_f32(float L, float T) { return sellmeier<float>(L, T); }
double oracle_n_f64(double L, double T) { return sellmeier<double>(L, T); }
float oracle_index_f32(int crystal, float L, float T) { return crystal_n<float>(crystal, L, T); }
double oracle_index_f64(int crystal, double L, double T) { return crystal_n<double>(crystal, L, T); }

void oracle_set_pump_f32(const oracle_cfg *c, float power, float focal, float waist, float tc, float *pump) {
    Model<float> m(*c);
    set_pump<float>(m, power, focal, waist, tc, as_cx(pump));
}
void oracle_set_pump_f64(const oracle_cfg *c, double power, double focal, double waist, double tc, double *pump) {
    Model<double> m(*c);
    set_pump<double>(m, power, focal, waist, tc, as_cx(pump));
}
void oracle_propagators_f32(const oracle_cfg *c, float tc, float *hp, float *hs) {
    Model<float> m(*c);
    propagators<float>(m, tc, as_cx(hp), as_cx(hs));
}
void oracle_propagators_f64(const oracle_cfg *c, double tc, double *hp, double *hs) {
    Model<double> m(*c);
    propagators<double>(m, tc, as_cx(hp), as_cx(hs));
}
float oracle_dk_constant_f32(const oracle_cfg *c, float temp) {
    Model<float> m(*c);
    return dk_constant<float>(m, temp);
}
double oracle_dk_constant_f64(const oracle_cfg *c, double temp) {
    Model<double> m(*c);
    return dk_constant<double>(m, temp);
}

void oracle_diffraction_f32(const oracle_cfg *c, float tc, float *pump, float *sh) {
    Model<float> m(*c);
    cvec<float> hp(m.NXY), hs(m.NXY), work;
    propagators<float>(m, tc, hp.data(), hs.data());
    diffraction<float>(m, hp.data(), hs.data(), as_cx(pump), as_cx(sh), work);
}

void oracle_dft2d_f32(int n0, int n1, int sign, const float *in, float *out) {
    dftref::dft2d<float>(in, out, n0, n1, sign);
}
void oracle_dft2d_f64(int n0, int n1, int sign, const double *in, double *out) {
    dftref::dft2d<double>(in, out, n0, n1, sign);
}

void oracle_cwes_plain_f32(const oracle_cfg *c, const float *pump, const float *sh, float temp, float dk,
                           float *out_pump, float *out_sh, float *end_pump, float *end_sh) {
    cwes_plain_impl<float>(c, pump, sh, temp, dk, out_pump, out_sh, end_pump, end_sh);
}
void oracle_cwes_plain_f64(const oracle_cfg *c, const double *pump, const double *sh, double temp, double dk,
                           double *out_pump, double *out_sh, double *end_pump, double *end_sh) {
    cwes_plain_impl<double>(c, pump, sh, temp, dk, out_pump, out_sh, end_pump, end_sh);
}

void oracle_run_plain_f32(const oracle_cfg *c, float power, float waist, float focal, float temp, int sh_seed,
                          float *out_pump, float *out_sh) {
    Model<float> m(*c);
    cvec<float> P(m.NXY), S(m.NXY, cx<float>{0.f, 0.f});
    set_pump<float>(m, power, focal, waist, temp, P.data());
    if (sh_seed >= 0) noise_f32(m.NXY, (unsigned)sh_seed, S.data());
    cvec<float> hp(m.NXY), hs(m.NXY);
    propagators<float>(m, temp, hp.data(), hs.data());
    const float dk = dk_constant<float>(m, temp);
    cwes<float>(m, P.data(), S.data(), hp.data(), hs.data(), false, dk, temp, nullptr, nullptr, nullptr,
                as_cx(out_pump), as_cx(out_sh));
}

void oracle_init_temperature(const oracle_cfg *c, float temp, float t1, float t2, int bc, float *T) {
    Model<float> m(*c);
    init_temperature(m, T, temp, t1, t2, bc);
}

void oracle_set_threads(int threads) { g_heat_threads = threads < 1 ? 1 : threads; }

// Tinic <- Tfinal after every sweep (Solver.h:321) is a swap of the two buffers here: the
// voxels a sweep never writes are equal in both, so the next sweep sees the same input.
void oracle_heat_sweeps(const oracle_cfg *c, float *T, const float *Q, float t_inf, int nsweeps, int bc) {
    Model<float> m(*c);
    HeatCoef hc(m);
    std::vector<float> Tf(T, T + m.TSIZE), Ti(T, T + m.TSIZE);
    for (int k = 0; k < nsweeps; ++k) {
        heat_sweep(m, hc, Tf.data(), Ti.data(), t_inf, Q, bc);
        std::swap(Ti, Tf);
    }
    std::memcpy(T, Ti.data(), m.TSIZE * sizeof(float));
}

float oracle_reduced_sum(const oracle_cfg *c, const float *Tf, const float *Ti) {
    Model<float> m(*c);
    return reduced_sum(m, Tf, Ti);
}

void oracle_dk_thermal(const oracle_cfg *c, const float *T, float *DK) {
    Model<float> m(*c);
    dk_thermal<float>(m, T, DK);
}

void oracle_cwes_thermal_f32(const oracle_cfg *c, const float *T, const float *DK3, const float *pump,
                             const float *sh, float tc, float *out_pump, float *out_sh) {
    cwes_thermal_impl<float>(c, T, DK3, pump, sh, tc, out_pump, out_sh);
}
void oracle_cwes_thermal_f64(const oracle_cfg *c, const double *T, const double *DK3, const double *pump,
                             const double *sh, double tc, double *out_pump, double *out_sh) {
    cwes_thermal_impl<double>(c, T, DK3, pump, sh, tc, out_pump, out_sh);
}

void oracle_set_q(const oracle_cfg *c, const float *T, const float *pump, const float *sh, int s, float *Q) {
    Model<float> m(*c);
    set_q<float>(m, Q, T, as_cx(pump), as_cx(sh), s);
}

int oracle_thermal_run(const oracle_cfg *c, float power, float waist, float focal, float temp, float t_inf,
                       float t1, float t2, int bc, int sh_seed, float *out_pump, float *out_sh, float *T_out,
                       int *counts) {
    Model<float> m(*c);
    HeatCoef hc(m);
    std::vector<float> Tf(m.TSIZE), Ti(m.TSIZE), Q(m.TSIZE, 0.0f), DK(m.TSIZE);
    init_temperature(m, Ti.data(), temp, t1, t2, bc);
    Tf = Ti;
    cvec<float> P(m.NXY), S(m.NXY), hp(m.NXY), hs(m.NXY);
    for (int i = 0; i < 5; ++i) counts[i] = -1;
    unsigned global_count = 0, num_of_iter = 5;
    int outer = 0;
    while (global_count < num_of_iter) {
        const float tol = (float)(5e-4 / (D)(unsigned)m.TSIZE);
        float Reduced_sum = 1.0f, aux_sum = -1.0f;
        unsigned counter_T = 0;
        while (Reduced_sum >= tol) {
            heat_sweep(m, hc, Tf.data(), Ti.data(), t_inf, Q.data(), bc);
            if (counter_T % 5000 == 0) {
                if (counter_T > 0) aux_sum = Reduced_sum;
                Reduced_sum = reduced_sum(m, Tf.data(), Ti.data());
                if (Reduced_sum == aux_sum) Reduced_sum = (float)(0.5 * (D)tol);
            }
            std::swap(Ti, Tf);  // Tinic <- Tfinal (Solver.h:321): both now hold the new field
            counter_T++;
        }
        Tf = Ti;
        counts[outer++] = (int)counter_T;
        dk_thermal<float>(m, Tf.data(), DK.data());
        const float tc = Tf[m.idx(m.NX / 2, m.NY / 2, 0)];
        set_pump<float>(m, power, focal, waist, tc, P.data());
        if (sh_seed >= 0)
            noise_f32(m.NXY, (unsigned)sh_seed, S.data());
        else
            std::fill(S.begin(), S.end(), cx<float>{0.f, 0.f});
        propagators<float>(m, tc, hp.data(), hs.data());
        cwes<float>(m, P.data(), S.data(), hp.data(), hs.data(), true, 0.0f, temp, Tf.data(), DK.data(),
                    Q.data(), as_cx(out_pump), as_cx(out_sh));
        if (counter_T == 1 && global_count != 0) global_count = num_of_iter;
        global_count++;
    }
    std::memcpy(T_out, Tf.data(), m.TSIZE * sizeof(float));
    return outer;
}

void oracle_sweep_plain(const oracle_cfg *crystal, const oracle_instance *inst, int n, int threads, double *eta) {
    std::atomic<int> next{0};
    auto worker = [&]() {
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n) break;
            oracle_cfg c = *crystal;
            c.nx = inst[i].nx;
            c.ny = inst[i].ny;
            c.nz = inst[i].nz;
            c.lx = inst[i].lx;
            c.ly = inst[i].ly;
            Model<float> m(c);
            std::vector<float> po(2 * m.NXY), so(2 * m.NXY), pin(2 * m.NXY);
            oracle_set_pump_f32(&c, inst[i].power, inst[i].focal, inst[i].waist, inst[i].temp, pin.data());
            oracle_run_plain_f32(&c, inst[i].power, inst[i].waist, inst[i].focal, inst[i].temp, -1, po.data(),
                                 so.data());
            const double pin_w = power_of<float>(m, as_cx((const float *)pin.data()), m.n(m.lp, inst[i].temp));
            const double psh = power_of<float>(m, as_cx((const float *)so.data()), m.n(m.ls, inst[i].temp));
            eta[i] = psh / pin_w;
        }
    };
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto &t : pool) t.join();
}

double oracle_power_f32(const oracle_cfg *c, const float *field, float n_index) {
    Model<float> m(*c);
    return power_of<float>(m, as_cx(field), n_index);
}

}  // extern "C"
