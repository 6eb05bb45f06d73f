// kg_hydro32.cu -- the FP32 form of the fused hydraulic operator.
//
// Same passes, block decomposition, tile-seam rules and stage formulas as k_hydro (the
// FP64 drop-in), with the arithmetic split by what needs FP64:
//   FP64  the free surface w and everything that subtracts a bed from it (cell depth
//         w - (b0+bt), the face offsets w - InterpolateB), the w and Hnpsi rows of the RHS
//         (flux differences of FP32 fluxes taken in FP64, so the sums over cells still
//         telescope and mass and solids are conserved to FP64 round-off), the w / Hnpsi
//         stage updates, the flux-source rates and the CFL minimum across CTAs;
//   FP32  reconstruction slopes, desingularised variables, wave speeds, the central-upwind
//         fluxes, hydrostatic and diffusive fluxes, momentum RHS rows, drag closures and
//         the momentum stage updates.
// Static geometric factors (gam, 1/gam, 1/gam^2, the hydrostatic prefactors, the face gam
// and wave-speed factor) come from the per-topography-set cache built by k_topo32, so a
// pass takes no FP64 divide or square root.  At rest (w flat, zero momenta) every face
// offset on both sides of a face is the same FP64 difference, so the state stays at rest.
#include <cuda_runtime.h>
#include "kg_engine.cuh"

namespace kg {

struct __align__(16) Hydro32Smem {
    double w[NR];                // free surface
    double p64[NR];              // Hnpsi as the stage update reads it
    float m1[NR], m2[NR], p[NR];
    float hp[NR], gam[NR], Hn[NR], rho[NR], u[NR], v[NR], psi[NR];
    float hlo[2][NLX], hhi[2][NLX];  // face-side depths w_face - InterpolateB at the cell's lower / upper
                                     // face (x, y), after the well-balancing correction
    float lx[5][NLX], ly[5][NLX];    // slopes of (-, Hnpsi, u, v, rho); row 0 (w) is not used
    float fx[7][NFX], fy[7][NFX];
    float red[NT / 32];
};

// Desingularised variables (src/HydraulicRHS.f90:762-878) in FP32 from the FP32 depth.
__device__ __forceinline__ void desing32(const DevParams32& P, float hp, float gam, float m1, float m2, float pp, float& Hn,
                                         float& psi, float& rho, float& u, float& v) {
    Hn = hp * gam;
    if (Hn < 0.f) Hn = 0.f;
    float Hnpsi = pp < 0.f ? 0.f : pp;
    float den = Hn * Hn + fmaxf(Hn * Hn, P.hThr2);
    float r2 = 2.f * Hn / den;
    psi = fminf(r2 * Hnpsi, P.maxPack);
    rho = density<float>(P, psi);
    float k = r2 / rho;
    u = k * m1;
    v = k * m2;
}

// (a - b) + (c - d) of four FP32 fluxes in FP64 with two conversions instead of four: the
// two differences and their sum are split error-free on the FP32 pipe (Knuth's TwoSum),
// the leading part and the summed error parts are converted and added.  The result is the
// exact sum to about 2^-47 relative (the FP32 rounding of the error sum), so the w and
// Hnpsi rows still telescope to FP64 round-off, and it is exactly 0 when the four fluxes
// cancel in pairs (a lake at rest).
__device__ __forceinline__ double flux_sum4(float a, float b, float c, float d) {
    float s1 = a - b, t = s1 - a, e1 = (a - (s1 - t)) + (-b - t);
    float s2 = c - d;
    t = s2 - c;
    float e2 = (c - (s2 - t)) + (-d - t);
    float S = s1 + s2;
    t = S - s1;
    float e3 = (s1 - (S - t)) + (s2 - t);
    float E = (e1 + e2) + e3;
    return (double)S + (double)E;
}

// Half of the limited free-surface difference (the step from a cell centre to its face,
// 0.5 dx * limiter(a/dx, b/dx) with a, b the forward and backward differences of w), in
// FP64.  On steep beds a thin flow's face depth is the small difference of two large
// terms, w - InterpolateB (metres) and this step (metres), so both stay in FP64 until the
// depth itself is formed.  The minmod family and the unlimited slope select or average
// the FP64 differences exactly as the limiters of src/Limiters.f90:68-184 do (the sign and
// magnitude tests are taken on the bit patterns); van Albada and WENO take their weight in
// FP32.
// x * 2^-k (k = 1, 2) on the integer pipe: the exponent field of a normal, finite double
// is lowered by k (exact); zeros, subnormals near the bottom and non-finite values take the
// FP64 multiply.
__device__ __forceinline__ double scale_down_pow2(double x, int k) {
    const int hi = __double2hiint(x);
    const int e = (hi >> 20) & 0x7FF;
    if (e > k && e < 0x7FF) return __hiloint2double(hi - (k << 20), __double2loint(x));
    return x * (k == 1 ? 0.5 : 0.25);
}

__device__ __forceinline__ double half_step_w(int lim, double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long ma = ia & 0x7FFFFFFFFFFFFFFFll, mb = ib & 0x7FFFFFFFFFFFFFFFll;
    switch (lim) {
        case KG_LIM_MINMOD1:
        case KG_LIM_MINMOD2: {
            if ((ia ^ ib) < 0 || ma == 0 || mb == 0) return 0.0;  // a * b <= 0
            const double m = ma < mb ? a : b;                    // the one nearer zero
            if (lim == KG_LIM_MINMOD1) return scale_down_pow2(m, 1);
            // min(theta a, theta b, (a + b)/2) of the same sign, halved (exactly: powers of 2)
            const double t1 = (0.5 * 1.3) * m, t2 = scale_down_pow2(a + b, 2);
            return (__double_as_longlong(t1) & 0x7FFFFFFFFFFFFFFFll) < (__double_as_longlong(t2) & 0x7FFFFFFFFFFFFFFFll) ? t1 : t2;
        }
        case KG_LIM_NONE: return scale_down_pow2(a + b, 2);
        default: return 0.5 * (double)limiter<float>(lim, (float)a, (float)b);
    }
}

// The two reconstructed face sides of a cell, as depths above the interpolated bed of each
// face (CorrectSlopes, src/HydraulicRHS.f90:560-735): dlo/dhi are w_c minus the bed of the
// lower/upper face, hs the half step of w.  A side below its bed corrects the cell: both
// sides then take w_c + (b_hi - b_lo)/2, i.e. (dlo + dhi)/2 above either face's bed.
// `corr_in` forces the correction (the ghost-tile rule, decided from stored records).
__device__ __forceinline__ void face_sides(double dlo, double dhi, double hs, int corr_in, float& lo, float& hi) {
    double up = dhi + hs, dn = dlo - hs;
    // x < 0 on the bit pattern (sign set, not -0): integer work instead of FP64 compares
    auto neg = [](double x) { long long b = __double_as_longlong(x); return b < 0 && b != (long long)0x8000000000000000ull; };
    bool corr = corr_in > 0 || (corr_in < 0 && (neg(up) || neg(dn)));
    if (corr) {
        float c = (float)(0.5 * (dlo + dhi));
        lo = c;
        hi = c;
    } else {
        lo = (float)dn;
        hi = (float)up;
    }
}

// The FP32 form stores the momenta in FP32: the state's momentum plane (plane 1 of a slot's
// four) holds rhoHnu as SC floats followed by rhoHnv as SC floats (plane 2 is unused); the
// momentum rows of ddtExplicit are packed the same way and ddtImplicit holds SC floats.
// The FP64 free surface and Hnpsi keep their planes.
__device__ __forceinline__ float* mom32(double* Q, int s, int SC) { return reinterpret_cast<float*>(Q + plane(s, 4, 1, SC)); }
__device__ __forceinline__ const float* mom32(const double* Q, int s, int SC) {
    return reinterpret_cast<const float*>(Q + plane(s, 4, 1, SC));
}
__device__ __forceinline__ float* imp32(double* I, int s, int SC) { return reinterpret_cast<float*>(I + plane(s, 1, 0, SC)); }
__device__ __forceinline__ const float* imp32(const double* I, int s, int SC) {
    return reinterpret_cast<const float*>(I + plane(s, 1, 0, SC));
}

struct Side32 {
    float hp, p, u, v, rho, du, dv;  // hp: face free surface minus InterpolateB at the face
};

// Central-upwind fluxes at one face in FP32 (CalculateFluxes, src/HydraulicRHS.f90:949-1064),
// written to out[k * stride] (the shared-memory flux rows).  gamf and kf = (1 + b_t^2)/gamf^3
// are the face's cached factors.
__device__ __forceinline__ void face_flux32(const DevParams32& P, bool xdir, const Side32& Pl, const Side32& Mi, float gamf,
                                            float kf, float gamL, float gamR, float h, float* out, int stride, float& cfl) {
    const float g = P.g;
    float HnP = Pl.hp * gamf, HnM = Mi.hp * gamf;
    float unP = xdir ? Pl.u : Pl.v, unM = xdir ? Mi.u : Mi.v;
    float hP = HnP <= 0.f ? 0.f : HnP, hM = HnM <= 0.f ? 0.f : HnM;
    float cP = sqrtf(g * hP * kf), cM = sqrtf(g * hM * kf);
    float aPos = fmaxf(fmaxf(unP + cP, unM + cM), 0.f);
    float aNeg = fminf(fminf(unP - cP, unM - cM), 0.f);
    if (aPos > 0.f) {
        float gr = fminf(gamL / gamf, 1.f);
        cfl = fminf(gr * gr * h / aPos, cfl);
    }
    if (aNeg < 0.f) {
        float gr = fminf(gamR / gamf, 1.f);
        cfl = fminf(gr * gr * h / -aNeg, cfl);
    }
    float dif = aPos - aNeg;
    if (dif < 1e-10f) {
#pragma unroll
        for (int k = 0; k < 7; ++k) out[k * stride] = 0.f;
        return;
    }
    float rdif = 1.f / dif;
    float ap = aPos * rdif, an = aNeg * rdif, apn = aPos * aNeg * rdif;
    float m1P = Pl.rho * HnP * Pl.u, m1M = Mi.rho * HnM * Mi.u;
    float m2P = Pl.rho * HnP * Pl.v, m2M = Mi.rho * HnM * Mi.v;
    out[0] = (HnP - HnM) * gamf * apn + gamf * (ap * HnM * unM - an * HnP * unP);
    out[3 * stride] = (Pl.p - Mi.p) * gamf * apn + gamf * (ap * Mi.p * unM - an * Pl.p * unP);
    out[stride] = (m1P - m1M) * apn + (ap * m1M * unM - an * m1P * unP);
    out[2 * stride] = (m2P - m2M) * apn + (ap * m2M * unM - an * m2P * unP);
    float GP = 0.5f * g * Pl.rho * Pl.hp * Pl.hp, GM = 0.5f * g * Mi.rho * Mi.hp * Mi.hp;
    out[4 * stride] = ap * GM - an * GP;
    const float nu = P.nu;
    float dP1 = 0.f, dP2 = 0.f, dM1 = 0.f, dM2 = 0.f;
    if (!(HnP < 0.f)) {
        dP1 = nu * Pl.rho * HnP * Pl.du;
        dP2 = nu * Pl.rho * HnP * Pl.dv;
    }
    if (!(HnM < 0.f)) {
        dM1 = nu * Mi.rho * HnM * Mi.du;
        dM2 = nu * Mi.rho * HnM * Mi.dv;
    }
    out[5 * stride] = 0.5f * (dP1 + dM1);
    out[6 * stride] = 0.5f * (dP2 + dM2);
}

// UpdateMaximum* on the state at the start of the step (src/TimeStepper.f90:519-524,
// :1155-1303) for cell c of a slot, in the last pass of a step.
__device__ __forceinline__ void update_maxima32(const DevArrays& A, const StepArgs& S, const StageTimes& Tm, const DevParams& P,
                                                const DevParams32& F, int slot, int c) {
    const int SC = P.nX * P.nY;
    const double* q0p = A.Q[S.q_tc] + plane(slot, 4, 0, SC) + c;
    const double* ct0 = A.CT[S.topo_tc] + plane(slot, 4, 0, SC) + c;
    double btt = ct0[SC];
    float bxt = (float)ct0[2 * (size_t)SC], byt = (float)ct0[3 * (size_t)SC];
    float gamt = gam_of<float>(P.geo, bxt, byt);
    float hpt = (float)((q0p[0] - ct0[0]) - btt);
    float Hn, psi, rho, u, v;
    const float* q0m = mom32(A.Q[S.q_tc], slot, SC);
    desing32(F, hpt, gamt, q0m[c], q0m[SC + c], (float)q0p[3 * (size_t)SC], Hn, psi, rho, u, v);
    double* M = A.MX + plane(slot, 11, 0, SC) + c;
    double tt = Tm.t_max;
    double Hnd = Hn, psid = psi;
    if (Hnd > P.hThr) {
        if (M[10 * (size_t)SC] == -1.0) M[10 * (size_t)SC] = tt;
        if (Hnd > M[0]) { M[0] = Hnd; M[(size_t)SC] = tt; }
    }
    double spd = sqrtf(modu2_of<float>(P.geo, u, v, bxt, byt));
    if ((spd > M[2 * (size_t)SC]) && (Hnd > P.hThr)) { M[2 * (size_t)SC] = spd; M[3 * (size_t)SC] = tt; }
    if (btt < 0.0 && -btt > M[4 * (size_t)SC]) { M[4 * (size_t)SC] = -btt; M[5 * (size_t)SC] = tt; }
    if (btt > 0.0 && btt > M[6 * (size_t)SC]) { M[6 * (size_t)SC] = btt; M[7 * (size_t)SC] = tt; }
    if (Hnd > P.hThr && psid > M[8 * (size_t)SC]) { M[8 * (size_t)SC] = psid; M[9 * (size_t)SC] = tt; }
}

// A dry block's pass (see hydro32_block): the RHS stage writes a zero RHS, the RK stages
// carry the block's input state (its own cells, as phase A loaded them) into their output
// buffer, and the last stage also stores the velocities and updates the running maxima.
__device__ __noinline__ void hydro32_dry_block(const DevArrays& A, const StepArgs& S, const StageTimes& Tm, const DevParams& P,
                                                  const DevParams32& F, const BlockDesc bd, const Hydro32Smem& sm) {
    const int nX = P.nX, SC = nX * P.nY;
    const int bx = min(BS, nX - bd.x0), by = min(BS, P.nY - bd.y0);
    const int tid = threadIdx.x, slot = bd.slot;
    if (tid >= bx * by) return;
    const int cx = tid % bx, cy = tid / bx, c = (bd.y0 + cy) * nX + (bd.x0 + cx);
    const int r = (cy + 2) * RG + (cx + 2);
    if (S.mode == MODE_RHS0) {
        double* Ed = A.E[S.e_set] + plane(slot, 4, 0, SC) + c;
        Ed[0] = 0.0;
        Ed[3 * (size_t)SC] = 0.0;
        float* Edm = mom32(A.E[S.e_set], slot, SC);
        Edm[c] = 0.f;
        Edm[SC + c] = 0.f;
        imp32(A.I[S.e_set], slot, SC)[c] = 0.f;
        return;
    }
    const int qo = S.mode == MODE_S1 ? S.q_s1 : S.mode == MODE_S2 ? S.q_s2 : S.q_out;
    double* dst = A.Q[qo] + plane(slot, 4, 0, SC) + c;
    dst[0] = sm.w[r];
    dst[3 * (size_t)SC] = sm.p64[r];
    float* dm = mom32(A.Q[qo], slot, SC);
    dm[c] = sm.m1[r];
    dm[SC + c] = sm.m2[r];
    if (S.mode == MODE_S3) {
        A.UV[plane(slot, 2, 0, SC) + c] = (double)sm.u[r];
        A.UV[plane(slot, 2, 1, SC) + c] = (double)sm.v[r];
        if (S.do_maxima) update_maxima32(A, S, Tm, P, F, slot, c);
    }
}

// One BS x BS block of one tile through one pass (the body shared by the single-simulation
// kernel, whose settings live in constant memory, and the batched kernel, whose settings
// come from a per-simulation table).
__device__ __forceinline__ void hydro32_block(const DevArrays& A, const StepArgs& S, const StageTimes& Tm, const DevParams& P,
                                              const DevParams32& F, const DevSource* src, const BlockDesc bd,
                                              Hydro32Smem& sm) {
    const int nX = P.nX, nY = P.nY, SC = nX * nY, SFX = (nX + 1) * nY, SFY = nX * (nY + 1);
    const int slot = bd.slot;
    const int bx = min(BS, nX - bd.x0), by = min(BS, nY - bd.y0);
    const int tid = threadIdx.x;
    const int nbW = A.nbr[slot * 8 + NB_W], nbE = A.nbr[slot * 8 + NB_E];
    const int nbN = A.nbr[slot * 8 + NB_N], nbS = A.nbr[slot * 8 + NB_S];
    const double* __restrict__ Qin = (S.mode == MODE_RHS0 || S.mode == MODE_S1) ? A.Q[S.q_in]
                                   : (S.mode == MODE_S2)                        ? A.Q[S.q_s1]
                                                                                : A.Q[S.q_s2];
    const double* __restrict__ TD = A.TD[S.topo];
    const float* __restrict__ TF = A.TF[S.topo];
    const double* __restrict__ FX = A.FX[S.topo];
    const double* __restrict__ FY = A.FY[S.topo];
    const float dtf = (float)Tm.dt;

    // ---- A: load the cross-shaped region, FP64 depth, FP32 desingularisation ----
    // `wet`: some region cell holds a depth, Hnpsi or momentum above F.dryEps (see below).
    bool wet = false;
    const float deps = F.dryEps;
    for (int r = tid; r < NR; r += NT) {
        int cx = r % RG - 2, cy = r / RG - 2;
        bool inX = (cy >= 0 && cy < by && cx >= -2 && cx < bx + 2);
        bool inY = (cx >= 0 && cx < bx && cy >= -2 && cy < by + 2);
        if (!inX && !inY) continue;
        int i = bd.x0 + cx, j = bd.y0 + cy, s = slot;
        if (i < 0) { s = nbW; i += nX; }
        else if (i >= nX) { s = nbE; i -= nX; }
        else if (j < 0) { s = nbS; j += nY; }
        else if (j >= nY) { s = nbN; j -= nY; }
        int c = j * nX + i;
        float gam = TF[plane(s, 6, 0, SC) + c];
        sm.gam[r] = gam;
        if (A.kind[s] == SLOT_GHOST) {
            double w = A.G9[plane(s, 9, 0, SC) + c], pp = A.G9[plane(s, 9, 3, SC) + c];
            sm.w[r] = w;
            sm.p64[r] = pp;
            sm.m1[r] = (float)A.G9[plane(s, 9, 1, SC) + c];
            sm.m2[r] = (float)A.G9[plane(s, 9, 2, SC) + c];
            sm.p[r] = (float)pp;
            sm.hp[r] = (float)(w - TD[plane(s, 3, 0, SC) + c]);
            sm.Hn[r] = (float)A.G9[plane(s, 9, 4, SC) + c];
            sm.u[r] = (float)A.G9[plane(s, 9, 5, SC) + c];
            sm.v[r] = (float)A.G9[plane(s, 9, 6, SC) + c];
            sm.psi[r] = (float)A.G9[plane(s, 9, 7, SC) + c];
            sm.rho[r] = (float)A.G9[plane(s, 9, 8, SC) + c];
            wet = wet || fabsf(sm.hp[r]) > deps || fabsf(sm.p[r]) > deps || fabsf(sm.m1[r]) > deps || fabsf(sm.m2[r]) > deps;
            continue;
        }
        double w, pp;
        float m1, m2;
        size_t q = plane(s, 4, 0, SC) + c;
        const float* Qm = mom32(Qin, s, SC);
        if (S.mode == MODE_S1) {
            // stage 1 on the fly (src/TimeStepper.f90:371-404): w, Hnpsi in FP64
            const double* E = A.E[S.e_set];
            const float* Em = mom32(E, s, SC);
            float I = imp32(A.I[S.e_set], s, SC)[c];
            w = Qin[q] + Tm.dt * E[q];
            pp = Qin[q + 3 * (size_t)SC] + Tm.dt * E[q + 3 * (size_t)SC];
            float den = 1.f / (1.f - dtf * I);
            m1 = (Qm[c] + dtf * Em[c]) * den;
            m2 = (Qm[SC + c] + dtf * Em[SC + c]) * den;
        } else {
            w = Qin[q];
            m1 = Qm[c];
            m2 = Qm[SC + c];
            pp = Qin[q + 3 * (size_t)SC];
        }
        float hp = (float)(w - TD[plane(s, 3, 0, SC) + c]);
        sm.w[r] = w; sm.p64[r] = pp; sm.m1[r] = m1; sm.m2[r] = m2; sm.p[r] = (float)pp; sm.hp[r] = hp;
        float Hn, psi, rho, u, v;
        desing32(F, hp, gam, m1, m2, (float)pp, Hn, psi, rho, u, v);
        sm.Hn[r] = Hn; sm.psi[r] = psi; sm.rho[r] = rho; sm.u[r] = u; sm.v[r] = v;
        wet = wet || fabsf(hp) > deps || fabsf(sm.p[r]) > deps || fabsf(m1) > deps || fabsf(m2) > deps;
    }
    // A dry block: no cell of the block or of its two-cell halo holds water (depth above
    // the bed, Hnpsi and both momenta all within dryEps = 1e-4 heightThreshold) and the tile
    // has no flux source.  Its faces then carry no flux beyond round-off of the bed
    // interpolation (face depths of order 1e-13 m, momentum fluxes of order 1e-26), its
    // closures are below the height threshold, and its cells' CFL terms exceed any dt, so
    // the pass carries the block's state forward with a zero RHS instead of running the
    // reconstruction, fluxes and RHS; the front of a flow is always at least two cells
    // away from such a block, and a flow moves less than a cell per pass (CFL <= 1).
    const bool src_tile = A.has_source[slot] != 0 && P.nSources >= 1;
    if (!__syncthreads_or(wet || src_tile)) {
        hydro32_dry_block(A, S, Tm, P, F, bd, sm);
        return;
    }

    // ---- B: limited slopes; reconstructed, corrected face-side depths of w in FP64 ----
    const int lim = P.limiter;
    const float dxR = F.dxR, dyR = F.dyR;
    for (int kk = tid; kk < (bx + 2) * by + (by + 2) * bx; kk += NT) {
        if (kk < (bx + 2) * by) {
            const int k = kk;
            int cx = k % (bx + 2) - 1, cy = k / (bx + 2);
            int r = (cy + 2) * RG + (cx + 2);
            int li = cy * (BS + 2) + (cx + 1);
            int i = bd.x0 + cx, j = bd.y0 + cy, s = slot;
            if (i < 0) { s = nbW; i += nX; }
            else if (i >= nX) { s = nbE; i -= nX; }
            const double* bI = FX + plane(s, 5, 4, SFX) + (size_t)j * (nX + 1) + i;
            const double dlo = sm.w[r] - bI[0], dhi = sm.w[r] - bI[1];
            bool ghW = (cx < 0 && bd.x0 == 0 && A.kind[nbW] == SLOT_GHOST);
            bool ghE = (cx >= bx && bd.x0 + bx == nX && A.kind[nbE] == SLOT_GHOST);
            double hs;
            int corr_in = -1;
            if (ghW || ghE) {
                // a ghost neighbour: its stored slope and stale face reconstructions decide
                const double* ge = A.GE + plane(ghW ? nbW : nbE, GE_COUNT, 0, A.nE);
                hs = ge[(ghW ? GE_LXN : GE_LX1) * A.nE + j] * (0.5 * P.dx);
                corr_in = ghW ? (ge[GE_MXN1 * A.nE + j] < bI[1] || ge[GE_PXN * A.nE + j] < bI[0])
                              : (ge[GE_MX2 * A.nE + j] < bI[1] || ge[GE_PX1 * A.nE + j] < bI[0]);
                sm.lx[1][li] = 0.f; sm.lx[2][li] = 0.f; sm.lx[3][li] = 0.f; sm.lx[4][li] = 0.f;
            } else {
                hs = half_step_w(lim, sm.w[r + 1] - sm.w[r], sm.w[r] - sm.w[r - 1]);
                sm.lx[1][li] = dxR * limiter<float>(lim, sm.p[r + 1] - sm.p[r], sm.p[r] - sm.p[r - 1]);
                sm.lx[2][li] = dxR * limiter<float>(lim, sm.u[r + 1] - sm.u[r], sm.u[r] - sm.u[r - 1]);
                sm.lx[3][li] = dxR * limiter<float>(lim, sm.v[r + 1] - sm.v[r], sm.v[r] - sm.v[r - 1]);
                sm.lx[4][li] = dxR * limiter<float>(lim, sm.rho[r + 1] - sm.rho[r], sm.rho[r] - sm.rho[r - 1]);
            }
            face_sides(dlo, dhi, hs, corr_in, sm.hlo[0][li], sm.hhi[0][li]);
        } else {
            const int k = kk - ((bx + 2) * by);
            int cx = k % bx, cy = k / bx - 1;
            int r = (cy + 2) * RG + (cx + 2);
            int li = (cy + 1) * BS + cx;
            int i = bd.x0 + cx, j = bd.y0 + cy, s = slot;
            if (j < 0) { s = nbS; j += nY; }
            else if (j >= nY) { s = nbN; j -= nY; }
            const double* bI = FY + plane(s, 5, 4, SFY) + (size_t)j * nX + i;
            const double dlo = sm.w[r] - bI[0], dhi = sm.w[r] - bI[nX];
            bool ghS = (cy < 0 && bd.y0 == 0 && A.kind[nbS] == SLOT_GHOST);
            bool ghN = (cy >= by && bd.y0 + by == nY && A.kind[nbN] == SLOT_GHOST);
            double hs;
            int corr_in = -1;
            if (ghS || ghN) {
                const double* ge = A.GE + plane(ghS ? nbS : nbN, GE_COUNT, 0, A.nE);
                hs = ge[(ghS ? GE_LYN : GE_LY1) * A.nE + i] * (0.5 * P.dy);
                corr_in = ghS ? (ge[GE_MYN1 * A.nE + i] < bI[nX] || ge[GE_PYN * A.nE + i] < bI[0])
                              : (ge[GE_MY2 * A.nE + i] < bI[nX] || ge[GE_PY1 * A.nE + i] < bI[0]);
                sm.ly[1][li] = 0.f; sm.ly[2][li] = 0.f; sm.ly[3][li] = 0.f; sm.ly[4][li] = 0.f;
            } else {
                hs = half_step_w(lim, sm.w[r + RG] - sm.w[r], sm.w[r] - sm.w[r - RG]);
                sm.ly[1][li] = dyR * limiter<float>(lim, sm.p[r + RG] - sm.p[r], sm.p[r] - sm.p[r - RG]);
                sm.ly[2][li] = dyR * limiter<float>(lim, sm.u[r + RG] - sm.u[r], sm.u[r] - sm.u[r - RG]);
                sm.ly[3][li] = dyR * limiter<float>(lim, sm.v[r + RG] - sm.v[r], sm.v[r] - sm.v[r - RG]);
                sm.ly[4][li] = dyR * limiter<float>(lim, sm.rho[r + RG] - sm.rho[r], sm.rho[r] - sm.rho[r - RG]);
            }
            face_sides(dlo, dhi, hs, corr_in, sm.hlo[1][li], sm.hhi[1][li]);
        }
    }
    __syncthreads();

    // ---- C: face states, corrections, fluxes, CFL ----
    float cfl = 3.402823466e38f;
    const float hdx = 0.5f * F.dx, hdy = 0.5f * F.dy;
    const float* __restrict__ TFXs = A.TFX[S.topo] + (size_t)slot * 2 * SFX;
    const float* __restrict__ TFYs = A.TFY[S.topo] + (size_t)slot * 2 * SFY;
    for (int kk = tid; kk < (bx + 1) * by + (by + 1) * bx; kk += NT) {
        if (kk < (bx + 1) * by) {
            const int k = kk;
            int fx = k % (bx + 1), cy = k / (bx + 1);
            int fi = bd.x0 + fx, j = bd.y0 + cy;
            int rL = (cy + 2) * RG + (fx + 1), rR = rL + 1;
            int liL = cy * (BS + 2) + fx, liR = liL + 1;
            Side32 L, R;
            // Left state: the upper-face reconstruction of cell fx-1.
            float sp = sm.lx[1][liL] * hdx;
            L.hp = sm.hhi[0][liL];
            L.p = sm.p[rL] + sp;
            if (L.p < 0.f || (fi != 0 && sm.p[rL] - sp < 0.f)) L.p = sm.p[rL];
            L.u = sm.u[rL] + sm.lx[2][liL] * hdx;
            L.v = sm.v[rL] + sm.lx[3][liL] * hdx;
            L.rho = sm.rho[rL] + sm.lx[4][liL] * hdx;
            L.du = sm.lx[2][liL];
            L.dv = sm.lx[3][liL];
            // Right state: the lower-face reconstruction of cell fx.
            sp = sm.lx[1][liR] * hdx;
            R.hp = sm.hlo[0][liR];
            R.p = sm.p[rR] - sp;
            if (R.p < 0.f || (fi != nX && sm.p[rR] + sp < 0.f)) R.p = sm.p[rR];
            R.u = sm.u[rR] - sm.lx[2][liR] * hdx;
            R.v = sm.v[rR] - sm.lx[3][liR] * hdx;
            R.rho = sm.rho[rR] - sm.lx[4][liR] * hdx;
            R.du = sm.lx[2][liR];
            R.dv = sm.lx[3][liR];
            int fo = j * (nX + 1) + fi;
            face_flux32(F, true, R, L, TFXs[fo], TFXs[fo + SFX], sm.gam[rL], sm.gam[rR], F.dx, &sm.fx[0][cy * (BS + 1) + fx], NFX, cfl);
        } else {
            const int k = kk - ((bx + 1) * by);
            int cx = k % bx, fy = k / bx;
            int fj = bd.y0 + fy, i = bd.x0 + cx;
            int rL = (fy + 1) * RG + (cx + 2), rR = rL + RG;
            int liL = fy * BS + cx, liR = liL + BS;
            Side32 L, R;
            float sp = sm.ly[1][liL] * hdy;
            L.hp = sm.hhi[1][liL];
            L.p = sm.p[rL] + sp;
            if (L.p < 0.f || (fj != 0 && sm.p[rL] - sp < 0.f)) L.p = sm.p[rL];
            L.u = sm.u[rL] + sm.ly[2][liL] * hdy;
            L.v = sm.v[rL] + sm.ly[3][liL] * hdy;
            L.rho = sm.rho[rL] + sm.ly[4][liL] * hdy;
            L.du = sm.ly[2][liL];
            L.dv = sm.ly[3][liL];
            sp = sm.ly[1][liR] * hdy;
            R.hp = sm.hlo[1][liR];
            R.p = sm.p[rR] - sp;
            if (R.p < 0.f || (fj != nY && sm.p[rR] + sp < 0.f)) R.p = sm.p[rR];
            R.u = sm.u[rR] - sm.ly[2][liR] * hdy;
            R.v = sm.v[rR] - sm.ly[3][liR] * hdy;
            R.rho = sm.rho[rR] - sm.ly[4][liR] * hdy;
            R.du = sm.ly[2][liR];
            R.dv = sm.ly[3][liR];
            int fo = fj * nX + i;
            face_flux32(F, false, R, L, TFYs[fo], TFYs[fo + SFY], sm.gam[rL], sm.gam[rR], F.dy, &sm.fy[0][fy * BS + cx], NFX, cfl);
        }
    }
    // CFL: warp then block min in FP32, the cross-CTA minimum on FP64 bits.
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cfl = fminf(cfl, __shfl_xor_sync(0xffffffffu, cfl, o));
    if ((tid & 31) == 0) sm.red[tid >> 5] = cfl;
    __syncthreads();
    if (tid == 0) {
        float m = sm.red[0];
        for (int q = 1; q < NT / 32; ++q) m = fminf(m, sm.red[q]);
        double md = m >= 3.402823466e38f ? 1.7976931348623157e308 : (double)m;
        atomicMin(S.cfl_min, (unsigned long long)__double_as_longlong(md));
    }

    // ---- D: RHS assembly and stage update for the block's own cells ----
    if (tid < bx * by) {
        int cx = tid % bx, cy = tid / bx;
        int i = bd.x0 + cx, j = bd.y0 + cy, c = j * nX + i;
        int r = (cy + 2) * RG + (cx + 2);
        const double* td = TD + plane(slot, 3, 0, SC) + c;
        const float* tf = TF + plane(slot, 6, 0, SC) + c;
        double ig2 = td[SC], ig = td[2 * (size_t)SC];
        float gam = tf[0], dbdx = tf[SC], dbdy = tf[2 * (size_t)SC];
        float gXp1 = tf[3 * (size_t)SC], gXp2 = tf[4 * (size_t)SC], gYp2 = tf[5 * (size_t)SC], gYp1 = gXp2;
        int xl = cy * (BS + 1) + cx, xr = xl + 1;
        int yb = cy * BS + cx, yt = yb + BS;
        // w and Hnpsi rows in FP64 (the flux differences of FP32 values are exact or nearly so)
        double E0, E3;
        if (__double_as_longlong(P.dx) == __double_as_longlong(P.dy)) {  // square cells (an integer test)
            // square cells: the four-flux sum once, from an error-free FP32 split
            E0 = flux_sum4(sm.fx[0][xl], sm.fx[0][xr], sm.fy[0][yb], sm.fy[0][yt]) * P.dxR * ig2;
            E3 = flux_sum4(sm.fx[3][xl], sm.fx[3][xr], sm.fy[3][yb], sm.fy[3][yt]) * P.dxR * ig;
        } else {
            E0 = (((double)sm.fx[0][xl] - (double)sm.fx[0][xr]) * P.dxR + ((double)sm.fy[0][yb] - (double)sm.fy[0][yt]) * P.dyR) * ig2;
            E3 = (((double)sm.fx[3][xl] - (double)sm.fx[3][xr]) * P.dxR + ((double)sm.fy[3][yb] - (double)sm.fy[3][yt]) * P.dyR) * ig;
        }
        float E1 = kahan3<float>(sm.fx[1][xl] - sm.fx[1][xr], (sm.fx[4][xl] - sm.fx[4][xr]) * gXp1, sm.fx[5][xr] - sm.fx[5][xl]) * dxR +
                   kahan3<float>(sm.fy[1][yb] - sm.fy[1][yt], (sm.fy[4][yb] - sm.fy[4][yt]) * gYp1, sm.fy[5][yt] - sm.fy[5][yb]) * dyR;
        float E2 = kahan3<float>(sm.fx[2][xl] - sm.fx[2][xr], (sm.fx[4][xl] - sm.fx[4][xr]) * gXp2, sm.fx[6][xr] - sm.fx[6][xl]) * dxR +
                   kahan3<float>(sm.fy[2][yb] - sm.fy[2][yt], (sm.fy[4][yb] - sm.fy[4][yt]) * gYp2, sm.fy[6][yt] - sm.fy[6][yb]) * dyR;
        // Sources (ExplicitSourceTerms, src/Equations.f90:456-620): flux sources in FP64,
        // gravity in FP32 from the FP64 depth.
        if (A.has_source[slot] != 0 && P.nSources >= 1) {
            int gi = (bd.tile - 1) % P.nXtiles + 1, gj = (bd.tile - 1) / P.nXtiles + 1;
            double x = -0.5 * P.xSize + P.dx * ((gi - 1.0) * P.nX + ((i + 1) - 0.5));
            double y = -0.5 * P.ySize + P.dy * ((gj - 1.0) * P.nY + ((j + 1) - 0.5));
            double s1 = 0.0, s3 = 0.0;
            flux_source_rates(P, src, Tm.t_rhs, S.t_grid, x, y, s1, s3);
            E0 = E0 + s1 * ig2;
            E3 = E3 + s3 * ig;
        }
        float grho = F.g * sm.rho[r] * sm.hp[r] / gam;
        E1 = E1 - grho * dbdx;
        E2 = E2 - grho * dbdy;
        Pt<float> pt{sm.Hn[r], sm.u[r], sm.v[r], sm.psi[r], sm.rho[r], 0.f, dbdx, dbdy, gam};
        float I = implicit_source<float>(F, pt, drag<float>(F, pt));
        if (S.mode == MODE_RHS0) {
            double* Ed = A.E[S.e_set] + plane(slot, 4, 0, SC) + c;
            Ed[0] = E0;
            float* Edm = mom32(A.E[S.e_set], slot, SC);
            Edm[c] = E1;
            Edm[SC + c] = E2;
            Ed[3 * (size_t)SC] = E3;
            imp32(A.I[S.e_set], slot, SC)[c] = I;
        } else if (S.mode == MODE_S1 || S.mode == MODE_S2) {
            const double* q0p = A.Q[S.q_in] + plane(slot, 4, 0, SC) + c;
            double b = td[0];
            double hp_old = q0p[0] - b, hp_new = sm.w[r] - b;
            double* dst = A.Q[S.mode == MODE_S1 ? S.q_s1 : S.q_s2] + plane(slot, 4, 0, SC) + c;
            float den = 1.f / (1.f - dtf * I);
            // stage weights (3/4, 1/4) and (1/3, 2/3); the FP32 copies are constants, and
            // the stage-2 quarter is an exact exponent shift on the integer pipe
            const bool s1 = S.mode == MODE_S1;
            const double a0 = s1 ? 0.75 : 1.0 / 3.0, a1 = s1 ? 0.25 : 2.0 / 3.0;
            const float a0f = s1 ? 0.75f : (float)(1.0 / 3.0), a1f = s1 ? 0.25f : (float)(2.0 / 3.0);
            const double wn = hp_new + Tm.dt * E0, pn = sm.p64[r] + Tm.dt * E3;
            dst[0] = b + (a0 * hp_old + (s1 ? scale_down_pow2(wn, 2) : a1 * wn));
            const float* q0m = mom32(A.Q[S.q_in], slot, SC);
            float* dm = mom32(A.Q[s1 ? S.q_s1 : S.q_s2], slot, SC);
            dm[c] = a0f * q0m[c] + a1f * (sm.m1[r] + dtf * E1) * den;
            dm[SC + c] = a0f * q0m[SC + c] + a1f * (sm.m2[r] + dtf * E2) * den;
            dst[3 * (size_t)SC] = a0 * q0p[3 * (size_t)SC] + (s1 ? scale_down_pow2(pn, 2) : a1 * pn);
        } else {
            float dt2I = dtf * dtf * I;
            float den = 1.f / (1.f + dt2I * I);
            double* dst = A.Q[S.q_out] + plane(slot, 4, 0, SC) + c;
            dst[0] = sm.w[r];
            float* dm = mom32(A.Q[S.q_out], slot, SC);
            dm[c] = (sm.m1[r] - dt2I * E1) * den;
            dm[SC + c] = (sm.m2[r] - dt2I * E2) * den;
            dst[3 * (size_t)SC] = sm.p64[r];
            A.UV[plane(slot, 2, 0, SC) + c] = (double)sm.u[r];
            A.UV[plane(slot, 2, 1, SC) + c] = (double)sm.v[r];
            if (S.do_maxima) update_maxima32(A, S, Tm, P, F, slot, c);
        }
    }
}

__global__ void __launch_bounds__(NT) k_hydro32(DevArrays A, const BlockDesc* __restrict__ blocks, const StepArgs S) {
    kg_dep_wait();
    StageTimes Tm;
    if (!stage_gate_open_warp(cP, S, Tm)) return;
    extern __shared__ __align__(16) unsigned char smraw[];
    Hydro32Smem& sm = *reinterpret_cast<Hydro32Smem*>(smraw);
    hydro32_block(A, S, Tm, cP, cP32, cSrc, blocks[blockIdx.x], sm);
}

// Topography factors of the FP32 form for the listed slots of set ts, from the FP64 cell
// and face topography (FP32 factors from FP32 slopes; 1/gam^2 and 1/gam to FP64 accuracy) (gam = sqrt(1 + b_x^2 + b_y^2), src/Closures.f90:174-186; the
// hydrostatic prefactors of ConstructHydraulicRHS, src/HydraulicRHS.f90:1236-1250; the
// wave-speed factor (1 + b_t^2)/gam^3 of src/Equations.f90:249-381).
__device__ __forceinline__ void topo32(const DevParams& P, const DevArrays& A, int s, int k, int ts) {
    const int nX = P.nX, nY = P.nY, SC = nX * nY, SFX = (nX + 1) * nY, SFY = nX * (nY + 1);
    if (k < SC) {
        const double* ct = A.CT[ts] + plane(s, 4, 0, SC) + k;
        double b0 = ct[0], bt = ct[SC], bx = ct[2 * (size_t)SC], by = ct[3 * (size_t)SC];
        double* td = A.TD[ts] + plane(s, 3, 0, SC) + k;
        float* tf = A.TF[ts] + plane(s, 6, 0, SC) + k;
        td[0] = b0 + bt;
        if (P.geo) {
            // 1/gam^2 and 1/gam to FP64 accuracy: FP32 seeds refined by two Newton steps.
            double g2 = 1.0 + (bx * bx + by * by);
            double r = (double)(1.f / (float)g2);
            r = r * (2.0 - g2 * r);
            r = r * (2.0 - g2 * r);
            double y = (double)rsqrtf((float)g2);
            y = y * (1.5 - 0.5 * g2 * y * y);
            y = y * (1.5 - 0.5 * g2 * y * y);
            td[SC] = r;
            td[2 * (size_t)SC] = y;
            float bxf = (float)bx, byf = (float)by, igf = (float)y;
            tf[0] = sqrtf((float)g2);
            tf[SC] = bxf;
            tf[2 * (size_t)SC] = byf;
            tf[3 * (size_t)SC] = (1.f + byf * byf) * igf;
            tf[4 * (size_t)SC] = -bxf * byf * igf;
            tf[5 * (size_t)SC] = (1.f + bxf * bxf) * igf;
        } else {
            td[SC] = 1.0;
            td[2 * (size_t)SC] = 1.0;
            tf[0] = 1.f;
            tf[SC] = (float)bx;
            tf[2 * (size_t)SC] = (float)by;
            tf[3 * (size_t)SC] = 1.f;
            tf[4 * (size_t)SC] = 0.f;
            tf[5 * (size_t)SC] = 1.f;
        }
    }
    if (k < SFX) {
        const double* fx = A.FX[ts] + plane(s, 5, 0, SFX) + k;
        float bx = (float)fx[2 * (size_t)SFX], by = (float)fx[3 * (size_t)SFX];
        float* o = A.TFX[ts] + plane(s, 2, 0, SFX) + k;
        float g = P.geo ? sqrtf(1.f + bx * bx + by * by) : 1.f;
        o[0] = g;
        o[SFX] = P.geo ? (1.f + by * by) / (g * g * g) : 1.f;
    }
    if (k < SFY) {
        const double* fy = A.FY[ts] + plane(s, 5, 0, SFY) + k;
        float bx = (float)fy[2 * (size_t)SFY], by = (float)fy[3 * (size_t)SFY];
        float* o = A.TFY[ts] + plane(s, 2, 0, SFY) + k;
        float g = P.geo ? sqrtf(1.f + bx * bx + by * by) : 1.f;
        o[0] = g;
        o[SFY] = P.geo ? (1.f + bx * bx) / (g * g * g) : 1.f;
    }
}

__global__ void __launch_bounds__(256) k_topo32(DevArrays A, const int* __restrict__ slots, int ts, int per) {
    kg_dep_wait();
    topo32(cP, A, slots[blockIdx.x / per], (blockIdx.x % per) * 256 + threadIdx.x, ts);
}

size_t hydro32_smem_bytes() { return sizeof(Hydro32Smem); }

cudaError_t launch_hydro32(const DevArrays& A, const BlockDesc* blocks, int nblocks, const StepArgs& S, cudaStream_t st) {
    // the shared-memory opt-in is a per-device function attribute: set once per device
    static bool attr[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!attr[dev]) {
        e = cudaFuncSetAttribute(k_hydro32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Hydro32Smem));
        if (e != cudaSuccess) return e;
        attr[dev] = true;
    }
    if (nblocks == 0) return cudaSuccess;
    KG_TRY_LAUNCH(kg_launch(k_hydro32, nblocks, NT, sizeof(Hydro32Smem), st, A, blocks, S));
    return cudaGetLastError();
}

cudaError_t launch_topo32(const DevArrays& A, const int* d_slots, int n, int ts, int nX, int nY, cudaStream_t st) {
    int items = (nX + 1) * (nY + 1);
    int per = (items + 255) / 256;
    if (n <= 0) return cudaSuccess;
    KG_TRY_LAUNCH(kg_launch(k_topo32, n * per, 256, 0, st, A, d_slots, ts, per));
    return cudaGetLastError();
}

}  // namespace kg
