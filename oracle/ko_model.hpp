// ko_model.hpp -- TEST INFRASTRUCTURE (the oracle), not part of the product.
//
// CPU FP64 restatement of Kestrel v1.1.1's time-step hot path, used only by tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline leg as the checker.  The product
// (kestrel_gb300/) never links, imports or executes anything under oracle/.
//
// Parity status: pinned against the reference's own invariant tests (tests/testlib.jl:
// conservation <= 1e-10, depth >= -1e-14, bt >= -EroDepth, lake-at-rest, tile-layout
// independence <= 1e-13 / 1e-11) run on the reference's own input files.  The reference
// ships no golden output vectors and cannot be compiled here (no Fortran compiler), so no
// field-by-field pin against the Fortran binary exists.
//
// This header holds the data model (src/Grid.f90:57-158, src/RunSettings.f90:161-340) and
// the point-wise physics (src/Closures.f90, src/Limiters.f90, src/Equations.f90).  Data
// are kept exactly as the reference keeps them: per tile, 13 fields with the field index
// fastest, per-tile vertex beds, face reconstructions and flux arrays, and five tile
// containers (tileContainer, intermed0..3) with deep-copy semantics.
//
// Arithmetic is written operand-for-operand in the Fortran order (left to right, no
// re-association) and compiled with -ffp-contract=off, so that the only differences to
// the reference's arithmetic are libm's last-bit behaviour and gfortran's FMA contraction.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <limits>
#include "../include/kestrel_gpu.h"

namespace ko {

// Variable indices, src/main.f90:116-141.
enum { iw = 1, irhoHnu = 2, irhoHnv = 3, iHnpsi = 4, iHn = 5, iu = 6, iv = 7, ipsi = 8,
       irho = 9, ib0 = 10, ibt = 11, idbdx = 12, idbdy = 13, ND = 13, NFLUX = 4 };
static const int IFLUX[4] = {1, 2, 3, 4};     // src/RunSettings.f90:351-355
static const int IDESING[5] = {5, 6, 7, 8, 9}; // src/RunSettings.f90:357-362

static const double EPS = std::numeric_limits<double>::epsilon();  // epsilon(1.0_wp)
static const double HUGE_ = std::numeric_limits<double>::max();    // huge(1.0_wp)
static const double PI = 3.141592653589793238462643383279502884;   // 4*atan(1.0_wp)

// 1-based Fortran-order arrays.
struct A3 {
    int n1 = 0, n2 = 0, n3 = 0;
    std::vector<double> v;
    bool allocated() const { return !v.empty(); }
    void allocate(int a, int b, int c, double init) { n1 = a; n2 = b; n3 = c; v.assign((size_t)a * b * c, init); }
    double& operator()(int a, int b, int c) { return v[(size_t)(a - 1) + (size_t)n1 * ((size_t)(b - 1) + (size_t)n2 * (size_t)(c - 1))]; }
    const double& operator()(int a, int b, int c) const { return v[(size_t)(a - 1) + (size_t)n1 * ((size_t)(b - 1) + (size_t)n2 * (size_t)(c - 1))]; }
    double* col(int b, int c) { return &(*this)(1, b, c); }
    const double* col(int b, int c) const { return &(*this)(1, b, c); }
};
struct A2 {
    int n1 = 0, n2 = 0;
    std::vector<double> v;
    bool allocated() const { return !v.empty(); }
    void allocate(int a, int b, double init) { n1 = a; n2 = b; v.assign((size_t)a * b, init); }
    double& operator()(int a, int b) { return v[(size_t)(a - 1) + (size_t)n1 * (size_t)(b - 1)]; }
    const double& operator()(int a, int b) const { return v[(size_t)(a - 1) + (size_t)n1 * (size_t)(b - 1)]; }
};

// TileType, src/Grid.f90:57-121.
struct Tile {
    bool TileOn = false, isGhostTile = false, containsSource = false;
    int neighbours[4] = {0, 0, 0, 0};   // W, E, N, S
    int cornertiles[4] = {0, 0, 0, 0};  // SW, SE, NW, NE
    int West() const { return neighbours[0]; }
    int East() const { return neighbours[1]; }
    int North() const { return neighbours[2]; }
    int South() const { return neighbours[3]; }
    std::vector<double> x, y, x_vertex, y_vertex;
    double xmin = 0, xmax = 0, ymin = 0, ymax = 0;
    A3 u;
    A2 b0, bt, EminusD;
    A3 Hnmax, umax, emax, dmax, psimax;
    A2 tfirst;
    A3 uLimX, uLimY, uPlusX, uMinusX, uPlusY, uMinusY;
    A3 hXFlux, hYFlux, gXFlux, gYFlux, pXFlux, pYFlux;
    A3 ddtExplicit, ddtImplicit;
    A2 ddtExplicitBt;
};

struct FluxSrc {
    double x, y, Radius;
    int nFluxSeries;
    std::vector<double> time, flux, psi;
    int NumCellsInSrc = 0;
};

// RunSet (src/RunSettings.f90:161-340) with derived quantities.
struct RunSet {
    kg_params p;
    int nXpertile, nYpertile, nXtiles, nYtiles, nTiles;
    double deltaX, deltaY, deltaXRecip, deltaYRecip, xSize, ySize, Xtilesize, Ytilesize;
    bool geometric_factors, MorphodynamicsOn, SpongeLayer;
    int bcs;
    double g, rhow, rhos, gred, Rep, ws0, nsettling, CriticalShields, diffusiveTimeScale;
    double heightThreshold, cfl, maxdt, tstart, tend, DeltaT;
    int TileBuffer, Nout;
    std::vector<FluxSrc> FluxSources;
    int nSources() const { return (int)FluxSources.size(); }
    double tan1deg;  // tan(pi/180), src/Closures.f90:600
};

// ---------------------------------------------------------------- Limiters.f90:83-184
inline double MinMod1(double a, double b) {
    if (a * b <= 0.0) return 0.0;
    if (a > 0.0) return std::min(a, b);
    return std::max(a, b);
}
inline double MinMod2(double a, double b) {
    const double theta = 1.3;
    if (a * b <= 0.0) return 0.0;
    if (a > 0.0) return std::min(theta * a, std::min(theta * b, 0.5 * (a + b)));
    return std::max(theta * a, std::max(theta * b, 0.5 * (a + b)));
}
inline double LimiterNone(double a, double b) { return 0.5 * (a + b); }
inline double vanAlbada(double a, double b) {
    double den = a * a + b * b;
    if (den == 0.0) return 0.0;
    return (a * a * b + a * b * b) / den;
}
inline double weno_func(double a) {
    const double eps = 1.0e-6;
    double epsaa = a * a + eps;
    return 1.0 / (epsaa * epsaa);
}
inline double WENO(double a, double b) {
    double wa = weno_func(a), wb = weno_func(b);
    return (wa * a + wb * b) / (wa + wb);
}
inline double limiter(const RunSet& rp, double a, double b) {
    switch (rp.p.limiter) {
        case KG_LIM_MINMOD1: return MinMod1(a, b);
        case KG_LIM_MINMOD2: return MinMod2(a, b);
        case KG_LIM_VANALBADA: return vanAlbada(a, b);
        case KG_LIM_WENO: return WENO(a, b);
        default: return LimiterNone(a, b);
    }
}

// ---------------------------------------------------------------- Closures.f90
// uv points at u(1:13) of one cell or face (uv[d-1] = u(d)).
inline double ComputeHn(double w, double b0, double bt, double gam) {  // :158-171
    double Hn = -bt;
    Hn = Hn + (w - b0);
    Hn = Hn * gam;
    return Hn;
}
inline double Gam(const RunSet& rp, const double* uv) {  // :269-300
    if (!rp.geometric_factors) return 1.0;
    double dbdx = uv[idbdx - 1], dbdy = uv[idbdy - 1];
    return std::sqrt(1.0 + dbdx * dbdx + dbdy * dbdy);
}
inline double Gam_gradin(const RunSet& rp, double dbdx, double dbdy) {
    if (!rp.geometric_factors) return 1.0;
    return std::sqrt(1.0 + dbdx * dbdx + dbdy * dbdy);
}
inline double FlowSquaredSpeedSlopeAligned(const RunSet& rp, const double* uv) {  // :178-203
    double dbdx = uv[idbdx - 1], dbdy = uv[idbdy - 1];
    double u = uv[iu - 1];
    double modu2;
    if (rp.geometric_factors) modu2 = u * u * (1.0 + dbdx * dbdx);
    else modu2 = u * u;
    double v = uv[iv - 1];
    if (rp.geometric_factors) modu2 = modu2 + v * v * (1.0 + dbdy * dbdy) + 2.0 * dbdx * dbdy * u * v;
    else modu2 = modu2 + v * v;
    return modu2;
}
inline double Density(const RunSet& rp, double psi) { return rp.rhow + (rp.rhos - rp.rhow) * psi; }

inline double PouliquenFrictionCoefficient(const RunSet& rp, double gcostheta, double Hn, double modu) {  // :441-464
    double mu1 = rp.p.PouliquenMinSlope, mu2 = rp.p.PouliquenMaxSlope, beta = rp.p.PouliquenBeta;
    if (Hn > rp.heightThreshold) {
        double Fr = modu / std::sqrt(gcostheta * Hn);
        double I = Fr * rp.p.SolidDiameter / Hn;
        return mu1 + (mu2 - mu1) * I / (beta + I);
    }
    return mu1;
}
// Test hook (off unless a test sets it through ko_set_closure_nudge): moves the result of
// every closure transcendental (pow, tanh, log, cos) by one ulp: up (mode +1), down (-1),
// or, for a mode >= 2, up, down or not at all per call from a pseudo-random sequence seeded
// by the mode.  The GPU calls CUDA's functions, which differ from glibc's in the last bits
// in either direction; the tests use the nudge to measure how far the reference's
// algorithm itself moves under such differences.
inline int& closure_nudge() {
    static int d = 0;
    return d;
}
inline uint64_t& closure_nudge_state() {
    static uint64_t x = 0;
    return x;
}
inline double nd(double v) {
    const int d = closure_nudge();
    if (d == 0) return v;
    int dir = d;
    if (d >= 2) {  // xorshift64
        uint64_t& x = closure_nudge_state();
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        dir = (int)(x % 3) - 1;
        if (dir == 0) return v;
    }
    return std::nextafter(v, dir > 0 ? HUGE_VAL : -HUGE_VAL);
}

inline double ChezyDrag(const RunSet& rp, const double* uv) {
    double modu2 = FlowSquaredSpeedSlopeAligned(rp, uv);
    return rp.p.ChezyCo * modu2;
}
inline double CoulombDrag(const RunSet& rp, const double* uv) {
    double Hn = uv[iHn - 1];
    double gam = Gam(rp, uv);
    double g = rp.g / gam;
    return rp.p.CoulombCo * g * Hn;
}
inline double PouliquenDrag(const RunSet& rp, const double* uv) {
    double Hn = uv[iHn - 1];
    double gam = Gam(rp, uv);
    double g = rp.g / gam;
    double modu2 = FlowSquaredSpeedSlopeAligned(rp, uv);
    double mu = PouliquenFrictionCoefficient(rp, g, Hn, std::sqrt(modu2));
    if (modu2 > 0) return mu * g * Hn;
    return 0.0;
}
inline double Edwards2019Drag(const RunSet& rp, const double* uv) {  // :471-506
    double Hn = uv[iHn - 1];
    double gam = Gam(rp, uv);
    double gperp = rp.g / gam;
    double modu = std::sqrt(FlowSquaredSpeedSlopeAligned(rp, uv));
    double Fr = modu / std::sqrt(gperp * Hn);
    double mu1 = rp.p.PouliquenMinSlope, mu2 = rp.p.PouliquenMaxSlope, mu3 = rp.p.PouliquenIntermediateSlope;
    double beta = rp.p.PouliquenBeta, betastar = rp.p.Edwards2019betastar, kappa = rp.p.Edwards2019kappa;
    double capgam = rp.p.Edwards2019Gamma, L = rp.p.SolidDiameter;
    double friction;
    if (Fr > betastar) {
        friction = mu1 + (mu2 - mu1) / (1.0 + Hn * beta / (L * (Fr + capgam)));
    } else {
        friction = (nd(std::pow(Fr / betastar, kappa))) *
                       (mu1 + (mu2 - mu1) / (1.0 + Hn * beta / (L * (betastar + capgam))) -
                        mu3 - (mu2 - mu1) / (1.0 + Hn / L)) +
                   mu3 + (mu2 - mu1) / (1.0 + Hn / L);
    }
    return friction * gperp * Hn;
}
inline double ManningDrag(const RunSet& rp, const double* uv) {  // :510-532
    double Hn = uv[iHn - 1];
    double gam = Gam(rp, uv);
    double g = rp.g / gam;
    double n = rp.p.ManningCo;
    if (Hn > rp.heightThreshold) return g * n * n / (nd(std::pow(Hn, 1.0 / 3.0)));
    return 0.0;
}
inline double fswitch(const RunSet& rp, double psi) {  // :797-915
    double rate = rp.p.VoellmySwitchRate, val = rp.p.VoellmySwitchValue;
    switch (rp.p.fswitch) {
        case KG_SWITCH_TANH: return 0.5 * (1.0 + nd(std::tanh(rate * (psi - val))));
        case KG_SWITCH_RAT3: {
            double a = val - 1.5 / rate, b = val + 1.5 / rate;
            if (psi <= a) return 0.0;
            if (psi >= b) return 1.0;
            double x = (psi - a) / (b - a);
            double omx = 1 - x;
            return (x * x * x) / (omx * omx * omx + x * x * x);
        }
        case KG_SWITCH_COS: {
            double a = val - 0.25 * PI / rate, b = val + 0.25 * PI / rate;
            if (psi <= a) return 0.0;
            if (psi >= b) return 1.0;
            double x = (psi - a) / (b - a);
            return 0.5 * (1.0 - nd(std::cos(PI * x)));
        }
        case KG_SWITCH_LINEAR: return psi / rp.p.maxPack;
        case KG_SWITCH_EQUAL: return 0.5;
        case KG_SWITCH_ZERO: return 0.0;
        case KG_SWITCH_ONE: return 1.0;
        default: return (psi < val) ? 0.0 : 1.0;  // step
    }
}
inline double VariableDrag(const RunSet& rp, const double* uv) {
    double psi = uv[ipsi - 1];
    double chezy_friction = ChezyDrag(rp, uv);
    double pouliquen_friction = PouliquenDrag(rp, uv);
    double fc = fswitch(rp, psi);
    return chezy_friction * (1.0 - fc) + pouliquen_friction * fc;
}
inline double DragClosure(const RunSet& rp, const double* uv) {
    switch (rp.p.drag) {
        case KG_DRAG_CHEZY: return ChezyDrag(rp, uv);
        case KG_DRAG_COULOMB: return CoulombDrag(rp, uv);
        case KG_DRAG_VOELLMY: return ChezyDrag(rp, uv) + CoulombDrag(rp, uv);
        case KG_DRAG_POULIQUEN: return PouliquenDrag(rp, uv);
        case KG_DRAG_EDWARDS2019: return Edwards2019Drag(rp, uv);
        case KG_DRAG_VARIABLE: return VariableDrag(rp, uv);
        default: return ManningDrag(rp, uv);
    }
}
inline double FlowShieldsNumber(const RunSet& rp, const double* uv) {  // :208-223
    double gred = rp.gred / Gam(rp, uv);
    double modu2 = FlowSquaredSpeedSlopeAligned(rp, uv);
    double chezy_friction = rp.p.ChezyCo * modu2;
    return chezy_friction / (gred * rp.p.SolidDiameter);
}
inline double FlowParticleSpeed(const RunSet& rp, const double* uv) {  // :228-240
    double gred = rp.gred / Gam(rp, uv);
    return std::sqrt(gred * rp.p.SolidDiameter);
}
inline double FluidErosion(const RunSet& rp, const double* uv) {  // :590-608
    double shields = FlowShieldsNumber(rp, uv);
    if (shields > rp.CriticalShields) {
        double ero = rp.p.EroRate * (shields - rp.CriticalShields);
        return ero * FlowParticleSpeed(rp, uv);
    }
    return 0.0;
}
inline double GranularErosion(const RunSet& rp, const double* uv) {  // :616-644
    double Hn = uv[iHn - 1];
    double modu2 = FlowSquaredSpeedSlopeAligned(rp, uv);
    double mu1 = rp.p.PouliquenMinSlope;
    double t1 = rp.tan1deg;
    double stat = (mu1 + t1) / (1.0 - mu1 * t1);
    double gcostheta = rp.g / Gam(rp, uv);
    double mu = PouliquenFrictionCoefficient(rp, gcostheta, Hn, std::sqrt(modu2));
    double q = Hn / 25.0 / rp.p.SolidDiameter;
    double muNeutral = mu1 + (stat - mu1) / (1.0 + q * q);
    if (mu > muNeutral) {
        double ero = rp.p.EroRateGranular * (mu - muNeutral);
        return ero * FlowParticleSpeed(rp, uv);
    }
    return 0.0;
}
inline double ErosionClosure(const RunSet& rp, const double* uv) {
    switch (rp.p.erosion) {
        case KG_ERO_MIXED: {
            double psi = uv[ipsi - 1];
            double fc = fswitch(rp, psi);
            double fluid_ero = FluidErosion(rp, uv);
            double granular_ero = GranularErosion(rp, uv);
            return (1.0 - fc) * fluid_ero + fc * granular_ero;
        }
        case KG_ERO_SIMPLE: {
            double shields = FlowShieldsNumber(rp, uv);
            double ero = rp.p.EroRate * shields;
            return ero * FlowParticleSpeed(rp, uv);
        }
        case KG_ERO_FLUID: return FluidErosion(rp, uv);
        case KG_ERO_GRANULAR: return GranularErosion(rp, uv);
        default: return 0.0;
    }
}
inline double ErosionTransition(const RunSet& rp, const double* uv) {  // :684-732
    double Bt = uv[ibt - 1];
    double eroDepth = rp.p.EroDepth;
    switch (rp.p.erosion_transition) {
        case KG_ETRANS_SMOOTH: return 0.5 * (1.0 + nd(std::tanh(1e5 * (Bt + eroDepth))));
        case KG_ETRANS_STEP: return (Bt < -eroDepth) ? 0.0 : 1.0;
        default: return 1.0;
    }
}
inline double MorphoDamping(const RunSet& rp, double Hn) {  // :744-791
    double Hncrit = rp.p.EroCriticalHeight;
    switch (rp.p.morpho_damping) {
        case KG_DAMP_TANH: return 0.5 * (1.0 + nd(std::tanh(10.0 * nd(std::log(Hn / Hncrit)))));
        case KG_DAMP_RAT3: {
            if (Hn < Hncrit) return 0.0;
            if (Hn > 2.0 * Hncrit) return 1.0;
            double t = Hn / Hncrit - 1.0;
            double omt = 1.0 - t;
            return (t * t * t) / (omt * omt * omt + t * t * t);
        }
        default: return 1.0;
    }
}
inline double DepositionClosure(const RunSet& rp, double psi) {  // :320-356
    switch (rp.p.deposition) {
        case KG_DEP_SIMPLE: return psi * (1.0 - psi / rp.p.maxPack);
        case KG_DEP_SPEARMAN_MANNING: {
            double a = 2.7 - 0.15 * rp.nsettling;
            double b = 0.62 * rp.nsettling - 1.46;
            return psi * nd(std::pow(1.0 - psi, a)) * nd(std::pow(1.0 - psi / rp.p.maxPack, b));
        }
        default: return 0.0;
    }
}

// ---------------------------------------------------------------- Equations.f90
inline void ErosionDepositionTerms(const RunSet& rp, const double* uv, double& E, double& D) {  // :385-405
    double Hn = uv[iHn - 1];
    E = ErosionClosure(rp, uv) * ErosionTransition(rp, uv);
    double psi = uv[ipsi - 1];
    double alpha;
    if (psi >= rp.p.maxPack) alpha = 0.0;
    else if (psi > 0.0) alpha = DepositionClosure(rp, psi);
    else alpha = 0.0;
    D = rp.ws0 * alpha;
    double damping = MorphoDamping(rp, Hn);
    E = E * damping;
    D = D * damping;
}

inline double XMaxWaveSpeeds(const RunSet& rp, const double* uv) {
    double Hn = uv[iHn - 1];
    if (Hn <= 0.0) Hn = 0.0;
    double u = uv[iu - 1];
    double gam = Gam(rp, uv);
    double by = uv[idbdy - 1];
    if (rp.geometric_factors) return u + std::sqrt(rp.g * Hn * (1.0 + by * by) / (gam * gam * gam));
    return u + std::sqrt(rp.g * Hn);
}
inline double XMinWaveSpeeds(const RunSet& rp, const double* uv) {
    double Hn = uv[iHn - 1];
    if (Hn <= 0.0) Hn = 0.0;
    double u = uv[iu - 1];
    double gam = Gam(rp, uv);
    double by = uv[idbdy - 1];
    if (rp.geometric_factors) return u - std::sqrt(rp.g * Hn * (1.0 + by * by) / (gam * gam * gam));
    return u - std::sqrt(rp.g * Hn);
}
inline double YMaxWaveSpeeds(const RunSet& rp, const double* uv) {
    double Hn = uv[iHn - 1];
    if (Hn <= 0.0) Hn = 0.0;
    double v = uv[iv - 1];
    double gam = Gam(rp, uv);
    double bx = uv[idbdx - 1];
    if (rp.geometric_factors) return v + std::sqrt(rp.g * Hn * (1.0 + bx * bx) / (gam * gam * gam));
    return v + std::sqrt(rp.g * Hn);
}
inline double YMinWaveSpeeds(const RunSet& rp, const double* uv) {
    double Hn = uv[iHn - 1];
    if (Hn <= 0.0) Hn = 0.0;
    double v = uv[iv - 1];
    double gam = Gam(rp, uv);
    double bx = uv[idbdx - 1];
    if (rp.geometric_factors) return v - std::sqrt(rp.g * Hn * (1.0 + bx * bx) / (gam * gam * gam));
    return v - std::sqrt(rp.g * Hn);
}
// Convection / hydrostatic / diffusion fluxes (:53-245), xf indexed 0..3 = (w, rhoHnu, rhoHnv, Hnpsi).
inline void XConvectionFlux(const RunSet& rp, const double* uv, double* xf) {
    double gam = Gam(rp, uv);
    xf[0] = uv[iHn - 1] * uv[iu - 1] * gam;
    xf[3] = uv[iHnpsi - 1] * uv[iu - 1] * gam;
    xf[1] = uv[irhoHnu - 1] * uv[iu - 1];
    xf[2] = uv[irhoHnv - 1] * uv[iu - 1];
}
inline void YConvectionFlux(const RunSet& rp, const double* uv, double* yf) {
    double gam = Gam(rp, uv);
    yf[0] = uv[iHn - 1] * uv[iv - 1] * gam;
    yf[3] = uv[iHnpsi - 1] * uv[iv - 1] * gam;
    yf[1] = uv[irhoHnu - 1] * uv[iv - 1];
    yf[2] = uv[irhoHnv - 1] * uv[iv - 1];
}
inline void HydrostaticFlux(const RunSet& rp, const double* uv, double* f) {
    f[0] = 0.0;
    f[3] = 0.0;
    double hp = -uv[ibt - 1];
    hp = hp + (uv[iw - 1] - uv[ib0 - 1]);
    f[1] = 0.5 * rp.g * uv[irho - 1] * hp * hp;
    f[2] = f[1];
}
inline void DiffusionFlux(const RunSet& rp, const double* uv, const double* du, double* f) {
    f[0] = 0.0;
    f[3] = 0.0;
    if (uv[iHn - 1] < 0.0) {
        f[1] = 0.0;
        f[2] = 0.0;
    } else {
        double nu = rp.p.EddyViscosity;
        f[1] = nu * uv[irho - 1] * uv[iHn - 1] * du[iu - 1];
        f[2] = nu * uv[irho - 1] * uv[iHn - 1] * du[iv - 1];
    }
}
// ImplicitSourceTerms (:627-658): the value written to both momentum rows.
inline double ImplicitMomentumSource(const RunSet& rp, const double* uv, double friction) {
    double Hn = uv[iHn - 1];
    if (Hn > rp.heightThreshold) {
        double modu = std::sqrt(FlowSquaredSpeedSlopeAligned(rp, uv));
        if (modu > 1.0e-8) {
            double hr = 1.0 / Hn;
            return -friction * hr / modu;
        }
    }
    return 0.0;
}

// utilities.f90:418-448
inline void KahanAdd(double x, double& s, double& c) {
    double y = x - c;
    double t = s + y;
    c = (t - s) - y;
    s = t;
}
inline double KahanSum(const double* a, int n) {
    double s = 0.0, c = 0.0;
    for (int i = 0; i < n; ++i) KahanAdd(a[i], s, c);
    return s;
}
template <int N>
inline double KahanSumL(const double (&a)[N]) { return KahanSum(a, N); }

}  // namespace ko
