// kg_physics.cuh -- point-wise physics of the hot path on the device.
//
// Closures (src/Closures.f90:158-915), limiters (src/Limiters.f90:83-184), wave speeds and
// fluxes (src/Equations.f90:53-658).  Every expression keeps the reference's operand order
// and the library is compiled with -fmad=false, so the FP64 form rounds exactly as the
// reference's arithmetic does wherever only +,-,*,/,sqrt are involved; tanh/log/pow/cos
// come from CUDA's math library (a few ulp from glibc's).
//
// The templates take a real type R: double for the FP64 drop-in, float for the flux and
// closure arithmetic of the FP32 form; the settings struct PP is DevParams or DevParams32.
#pragma once
#include <cstdint>
#include "../../include/kestrel_gpu.h"

#define KG_HD __host__ __device__ __forceinline__

namespace kg {

// Run settings the kernels read, derived on the host from kg_params
// (src/Parameters.f90:629-648, src/DomainSettings.f90:185-225).
struct DevParams {
    int nX, nY, nXtiles, nYtiles;
    double dx, dy, dxR, dyR, xSize, ySize;
    int geo, morpho, drag, erosion, deposition, etrans, damping, fswitch, limiter, bcs;
    int TileBuffer, nSources;
    double g, rhow, rhos, gred, ws0, nsettling, CriticalShields;
    double ChezyCo, ManningCo, CoulombCo;
    double PMin, PMax, PInt, PBeta, Ebetastar, Ekappa, EGamma;
    double SwRate, SwValue;
    double EroRate, EroRateGranular, EroDepth, EroCriticalHeight, BedPorosity;
    double maxPack, SolidDiameter, nu, hThr, tan1deg, SpongeStrength;
    double cfl, maxdt, diffusiveTimeScale;
    double invSolid;  // 1 / (1 - BedPorosity), for the FP32 form's multiplications
    double hdxR, hdyR;  // 0.5 / dx, 0.5 / dy
    int no_dry_skip;    // FP32 form: run every block of a pass in full (kg_set_dry_skip(ctx, 0))
};

// The same settings in FP32 for the FP32 form's arithmetic (a conversion from FP64 is an
// FP64-pipe instruction on this GPU, so FP32 code reads these instead), plus hThr^2.
#define KG_PARAMS_REALS(X)                                                                                          \
    X(dx) X(dy) X(dxR) X(dyR) X(xSize) X(ySize) X(g) X(rhow) X(rhos) X(gred) X(ws0) X(nsettling) X(CriticalShields) \
    X(ChezyCo) X(ManningCo) X(CoulombCo) X(PMin) X(PMax) X(PInt) X(PBeta) X(Ebetastar) X(Ekappa) X(EGamma)         \
    X(SwRate) X(SwValue) X(EroRate) X(EroRateGranular) X(EroDepth) X(EroCriticalHeight) X(BedPorosity) X(maxPack)   \
    X(SolidDiameter) X(nu) X(hThr) X(tan1deg) X(SpongeStrength) X(cfl) X(maxdt) X(diffusiveTimeScale)
#define KG_PARAMS_INTS(X)                                                                                           \
    X(nX) X(nY) X(nXtiles) X(nYtiles) X(geo) X(morpho) X(drag) X(erosion) X(deposition) X(etrans) X(damping)       \
    X(fswitch) X(limiter) X(bcs) X(TileBuffer) X(nSources)
struct DevParams32 {
#define KG_F(n) float n;
#define KG_I(n) int n;
    KG_PARAMS_REALS(KG_F)
    KG_PARAMS_INTS(KG_I)
#undef KG_F
#undef KG_I
    float hThr2;
    float dryEps;  // FP32 form: depth, Hnpsi and momentum magnitude below which a block counts as dry
};
inline DevParams32 params32(const DevParams& d) {
    DevParams32 f{};
#define KG_F(n) f.n = (float)d.n;
#define KG_I(n) f.n = d.n;
    KG_PARAMS_REALS(KG_F)
    KG_PARAMS_INTS(KG_I)
#undef KG_F
#undef KG_I
    f.hThr2 = (float)(d.hThr * d.hThr);
    f.dryEps = d.no_dry_skip ? -1.f : (float)(1e-4 * d.hThr);  // -1: no block counts as dry
    return f;
}

constexpr double kPI = 3.141592653589793238462643383279502884;
constexpr double kEPS = 2.220446049250313080847263336181640625e-16;  // epsilon(1.0_wp)

// Fortran MIN/MAX as std::min/std::max evaluate them (first argument on ties).
template <class R> KG_HD R mn(R a, R b) { return (b < a) ? b : a; }
template <class R> KG_HD R mx(R a, R b) { return (a < b) ? b : a; }

template <class R> KG_HD R limiter(int which, R a, R b) {
    switch (which) {
        case KG_LIM_MINMOD1:
            if (a * b <= R(0)) return R(0);
            return (a > R(0)) ? mn(a, b) : mx(a, b);
        case KG_LIM_MINMOD2: {
            const R theta = R(1.3);
            if (a * b <= R(0)) return R(0);
            if (a > R(0)) return mn(theta * a, mn(theta * b, R(0.5) * (a + b)));
            return mx(theta * a, mx(theta * b, R(0.5) * (a + b)));
        }
        case KG_LIM_VANALBADA: {
            R den = a * a + b * b;
            if (den == R(0)) return R(0);
            return (a * a * b + a * b * b) / den;
        }
        case KG_LIM_WENO: {
            R ea = a * a + R(1.0e-6), eb = b * b + R(1.0e-6);
            R wa = R(1) / (ea * ea), wb = R(1) / (eb * eb);
            return (wa * a + wb * b) / (wa + wb);
        }
        default: return R(0.5) * (a + b);
    }
}

template <class R> KG_HD R gam_of(int geo, R dbdx, R dbdy) {
    if (!geo) return R(1);
    return sqrt(R(1) + dbdx * dbdx + dbdy * dbdy);
}
// ComputeHn, src/Closures.f90:158-171: the bed is removed in two steps.
template <class R> KG_HD R compute_hn(R w, R b0, R bt, R gam) {
    R Hn = -bt;
    Hn = Hn + (w - b0);
    return Hn * gam;
}
template <class R> KG_HD R modu2_of(int geo, R u, R v, R dbdx, R dbdy) {
    R m;
    if (geo) m = u * u * (R(1) + dbdx * dbdx);
    else m = u * u;
    if (geo) m = m + v * v * (R(1) + dbdy * dbdy) + R(2) * dbdx * dbdy * u * v;
    else m = m + v * v;
    return m;
}
template <class R, class PP> KG_HD R density(const PP& P, R psi) { return R(P.rhow) + (R(P.rhos) - R(P.rhow)) * psi; }

// Cell / face state the closures read (a subset of the reference's 13-vector).
template <class R> struct Pt {
    R Hn, u, v, psi, rho, bt, dbdx, dbdy, gam;
};

// 0.5 (1 + tanh x), the smooth switch of several closures.  The FP64 form evaluates the
// reference's expression; the FP32 form uses the equal logistic 1 / (1 + exp(-2x)), which
// keeps its relative precision where 1 + tanh x cancels (x below about -9 in FP32).
template <class R> KG_HD R half_one_plus_tanh(R x) { return R(0.5) * (R(1) + tanh(x)); }
template <> KG_HD float half_one_plus_tanh<float>(float x) { return 1.f / (1.f + expf(-2.f * x)); }

template <class R, class PP> KG_HD R pouliquen_mu(const PP& P, R gcos, R Hn, R modu) {
    R mu1 = R(P.PMin), mu2 = R(P.PMax), beta = R(P.PBeta);
    if (Hn > R(P.hThr)) {
        R Fr = modu / sqrt(gcos * Hn);
        R I = Fr * R(P.SolidDiameter) / Hn;
        return mu1 + (mu2 - mu1) * I / (beta + I);
    }
    return mu1;
}
template <class R, class PP> KG_HD R fswitch(const PP& P, R psi) {
    R rate = R(P.SwRate), val = R(P.SwValue);
    switch (P.fswitch) {
        case KG_SWITCH_TANH: return half_one_plus_tanh<R>(rate * (psi - val));
        case KG_SWITCH_RAT3: {
            R a = val - R(1.5) / rate, b = val + R(1.5) / rate;
            if (psi <= a) return R(0);
            if (psi >= b) return R(1);
            R x = (psi - a) / (b - a), o = R(1) - x;
            return (x * x * x) / (o * o * o + x * x * x);
        }
        case KG_SWITCH_COS: {
            R a = val - R(0.25) * R(kPI) / rate, b = val + R(0.25) * R(kPI) / rate;
            if (psi <= a) return R(0);
            if (psi >= b) return R(1);
            R x = (psi - a) / (b - a);
            return R(0.5) * (R(1) - cos(R(kPI) * x));
        }
        case KG_SWITCH_LINEAR: return psi / R(P.maxPack);
        case KG_SWITCH_EQUAL: return R(0.5);
        case KG_SWITCH_ZERO: return R(0);
        case KG_SWITCH_ONE: return R(1);
        default: return (psi < val) ? R(0) : R(1);
    }
}
template <class R, class PP> KG_HD R chezy(const PP& P, const Pt<R>& s) {
    return R(P.ChezyCo) * modu2_of(P.geo, s.u, s.v, s.dbdx, s.dbdy);
}
template <class R, class PP> KG_HD R coulomb(const PP& P, const Pt<R>& s) {
    R g = R(P.g) / s.gam;
    return R(P.CoulombCo) * g * s.Hn;
}
template <class R, class PP> KG_HD R pouliquen(const PP& P, const Pt<R>& s) {
    R g = R(P.g) / s.gam;
    R m2 = modu2_of(P.geo, s.u, s.v, s.dbdx, s.dbdy);
    R mu = pouliquen_mu(P, g, s.Hn, sqrt(m2));
    if (m2 > R(0)) return mu * g * s.Hn;
    return R(0);
}
// DragClosure dispatch (src/Parameters.f90:222-247).
template <class R, class PP> KG_HD R drag(const PP& P, const Pt<R>& s) {
    switch (P.drag) {
        case KG_DRAG_CHEZY: return chezy(P, s);
        case KG_DRAG_COULOMB: return coulomb(P, s);
        case KG_DRAG_VOELLMY: return chezy(P, s) + coulomb(P, s);
        case KG_DRAG_POULIQUEN: return pouliquen(P, s);
        case KG_DRAG_EDWARDS2019: {
            R gperp = R(P.g) / s.gam;
            R modu = sqrt(modu2_of(P.geo, s.u, s.v, s.dbdx, s.dbdy));
            R Fr = modu / sqrt(gperp * s.Hn);
            R mu1 = R(P.PMin), mu2 = R(P.PMax), mu3 = R(P.PInt), beta = R(P.PBeta);
            R bs = R(P.Ebetastar), L = R(P.SolidDiameter), cg = R(P.EGamma), Hn = s.Hn;
            R f;
            if (Fr > bs) {
                f = mu1 + (mu2 - mu1) / (R(1) + Hn * beta / (L * (Fr + cg)));
            } else {
                f = (pow(Fr / bs, R(P.Ekappa))) *
                        (mu1 + (mu2 - mu1) / (R(1) + Hn * beta / (L * (bs + cg))) - mu3 - (mu2 - mu1) / (R(1) + Hn / L)) +
                    mu3 + (mu2 - mu1) / (R(1) + Hn / L);
            }
            return f * gperp * Hn;
        }
        case KG_DRAG_VARIABLE: {
            R c = chezy(P, s), p = pouliquen(P, s), fc = fswitch(P, s.psi);
            return c * (R(1) - fc) + p * fc;
        }
        default: {  // Manning: g n^2 / Hn^(1/3), no |u|^2 factor (src/Closures.f90:510-532)
            R g = R(P.g) / s.gam;
            R n = R(P.ManningCo);
            if (s.Hn > R(P.hThr)) return g * n * n / (pow(s.Hn, R(1) / R(3)));
            return R(0);
        }
    }
}
// ImplicitSourceTerms (src/Equations.f90:627-658): the value of both momentum rows.
template <class R, class PP> KG_HD R implicit_source(const PP& P, const Pt<R>& s, R friction) {
    if (s.Hn > R(P.hThr)) {
        R modu = sqrt(modu2_of(P.geo, s.u, s.v, s.dbdx, s.dbdy));
        if (modu > R(1.0e-8)) {
            R hr = R(1) / s.Hn;
            return -friction * hr / modu;
        }
    }
    return R(0);
}

// -- erosion / deposition (src/Closures.f90:566-791, src/Equations.f90:385-448) --
template <class R, class PP> KG_HD R shields(const PP& P, const Pt<R>& s) {
    R gred = R(P.gred) / s.gam;
    R cf = R(P.ChezyCo) * modu2_of(P.geo, s.u, s.v, s.dbdx, s.dbdy);
    return cf / (gred * R(P.SolidDiameter));
}
template <class R, class PP> KG_HD R particle_speed(const PP& P, const Pt<R>& s) {
    R gred = R(P.gred) / s.gam;
    return sqrt(gred * R(P.SolidDiameter));
}
template <class R, class PP> KG_HD R fluid_erosion(const PP& P, const Pt<R>& s) {
    R sh = shields(P, s);
    if (sh > R(P.CriticalShields)) {
        R ero = R(P.EroRate) * (sh - R(P.CriticalShields));
        return ero * particle_speed(P, s);
    }
    return R(0);
}
template <class R, class PP> KG_HD R granular_erosion(const PP& P, const Pt<R>& s) {
    R m2 = modu2_of(P.geo, s.u, s.v, s.dbdx, s.dbdy);
    R mu1 = R(P.PMin), t1 = R(P.tan1deg);
    R stat = (mu1 + t1) / (R(1) - mu1 * t1);
    R gcos = R(P.g) / s.gam;
    R mu = pouliquen_mu(P, gcos, s.Hn, sqrt(m2));
    R q = s.Hn / R(25) / R(P.SolidDiameter);
    R muN = mu1 + (stat - mu1) / (R(1) + q * q);
    if (mu > muN) {
        R ero = R(P.EroRateGranular) * (mu - muN);
        return ero * particle_speed(P, s);
    }
    return R(0);
}
template <class R, class PP> KG_HD R erosion_closure(const PP& P, const Pt<R>& s) {
    switch (P.erosion) {
        case KG_ERO_MIXED: {
            R fc = fswitch(P, s.psi);
            R fe = fluid_erosion(P, s), ge = granular_erosion(P, s);
            return (R(1) - fc) * fe + fc * ge;
        }
        case KG_ERO_SIMPLE: {
            R ero = R(P.EroRate) * shields(P, s);
            return ero * particle_speed(P, s);
        }
        case KG_ERO_FLUID: return fluid_erosion(P, s);
        case KG_ERO_GRANULAR: return granular_erosion(P, s);
        default: return R(0);
    }
}
template <class R, class PP> KG_HD R erosion_transition(const PP& P, R bt) {
    R d = R(P.EroDepth);
    switch (P.etrans) {
        case KG_ETRANS_SMOOTH: return half_one_plus_tanh<R>(R(1e5) * (bt + d));
        case KG_ETRANS_STEP: return (bt < -d) ? R(0) : R(1);
        default: return R(1);
    }
}
template <class R, class PP> KG_HD R morpho_damping(const PP& P, R Hn) {
    R Hc = R(P.EroCriticalHeight);
    switch (P.damping) {
        case KG_DAMP_TANH: return half_one_plus_tanh<R>(R(10) * log(Hn / Hc));
        case KG_DAMP_RAT3: {
            if (Hn < Hc) return R(0);
            if (Hn > R(2) * Hc) return R(1);
            R t = Hn / Hc - R(1), o = R(1) - t;
            return (t * t * t) / (o * o * o + t * t * t);
        }
        default: return R(1);
    }
}
template <class R, class PP> KG_HD R deposition_closure(const PP& P, R psi) {
    switch (P.deposition) {
        case KG_DEP_SIMPLE: return psi * (R(1) - psi / R(P.maxPack));
        case KG_DEP_SPEARMAN_MANNING: {
            R a = R(2.7) - R(0.15) * R(P.nsettling);
            R b = R(0.62) * R(P.nsettling) - R(1.46);
            return psi * pow(R(1) - psi, a) * pow(R(1) - psi / R(P.maxPack), b);
        }
        default: return R(0);
    }
}
// E - D with damping (ErosionDepositionTerms, src/Equations.f90:385-405).
template <class R, class PP> KG_HD R erosion_minus_deposition(const PP& P, const Pt<R>& s) {
    R E = erosion_closure(P, s) * erosion_transition(P, s.bt);
    R alpha;
    if (s.psi >= R(P.maxPack)) alpha = R(0);
    else if (s.psi > R(0)) alpha = deposition_closure(P, s.psi);
    else alpha = R(0);
    R D = R(P.ws0) * alpha;
    R damping = morpho_damping(P, s.Hn);
    E = E * damping;
    D = D * damping;
    return E - D;
}

// KahanAdd, src/utilities.f90:439-448.
template <class R> KG_HD void kahan_add(R x, R& s, R& c) {
    R y = x - c;
    R t = s + y;
    c = (t - s) - y;
    s = t;
}
template <class R> KG_HD R kahan3(R a, R b, R c) {
    R s = R(0), k = R(0);
    kahan_add(a, s, k);
    kahan_add(b, s, k);
    kahan_add(c, s, k);
    return s;
}
template <class R> KG_HD R kahan4(R a, R b, R c, R d) {
    R s = R(0), k = R(0);
    kahan_add(a, s, k);
    kahan_add(b, s, k);
    kahan_add(c, s, k);
    kahan_add(d, s, k);
    return s;
}
template <class R> KG_HD R kahan8(const R* a) {
    R s = R(0), k = R(0);
#pragma unroll
    for (int i = 0; i < 8; ++i) kahan_add(a[i], s, k);
    return s;
}
// InterpolateB, src/HydraulicRHS.f90:741-753.
template <class R> KG_HD R interp_b(R b0_0, R b0_1, R bt_0, R bt_1) {
    R b = bt_0 + bt_1;
    b = b + b0_0;
    b = b + b0_1;
    return b * R(0.5);
}

}  // namespace kg
