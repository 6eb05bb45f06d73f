// kg_hydro.cu -- fused FP64 hydraulic operator and RK stages on sm_103a.
//
// One CTA advances one BS x BS block of one active tile through one hydraulic RHS
// evaluation (CalculateHydraulicRHS, src/HydraulicRHS.f90:64-136) and, where the stage dt
// is already known, the RK update that consumes it (HydraulicTimeStepper,
// src/TimeStepper.f90:333-527):
//   MODE_RHS0  RHS(q0)                          -> E0, I0           (substep 1)
//   MODE_S1    q1 = stage1(q0,E0,I0) on the fly, RHS(q1) -> q2      (substep 2)
//   MODE_S2    RHS(q2)                          -> q3                (substep 3)
//   MODE_S3    RHS(q3), final implicit drag step -> q_new, maxima    (substep 4)
// Each pass also reduces the CFL terms of its faces (ComputeAdvisedTimeStep's input) into a
// single ordered-bits atomicMin.
//
// The seven per-tile phases of the reference become five in-CTA phases over a cross-shaped
// region of the block plus two halo cells in x and y:
//   A  load q and cell topography, desingularise (ComputeDesingularisedVariables)
//   B  limited slopes of w, Hnpsi, u, v, rho (CalculateLimitedDerivs; the other fields'
//      slopes and face values are overwritten in the reference before they are read)
//   C  face states with the well-balancing/positivity corrections (Reconstruct,
//      CorrectSlopes) and central-upwind fluxes + CFL terms (CalculateFluxes)
//   D  flux differences, sources, drag and the stage update (ConstructHydraulicRHS)
// Tile seams follow the reference's per-tile view: a tile's seam face takes the
// neighbour's corrected w (active neighbour) or applies the correction test to the ghost
// tile's stored reconstructions (ghost neighbour), and its Hnpsi is only reset when the
// reconstructed value itself is negative (src/HydraulicRHS.f90:597-614, :655-666).
#include <cuda_runtime.h>
#include "kg_engine.cuh"

namespace kg {

__constant__ DevParams cP;
__constant__ DevParams32 cP32;  // FP32 copy for the FP32 form
__constant__ DevSource cSrc[MAX_SRC];

constexpr int BS = 16;
constexpr int RG = BS + 4;
constexpr int NT = BS * BS;
constexpr int NR = RG * RG;
constexpr int NLX = (BS + 2) * BS;
constexpr int NFX = (BS + 1) * BS;

struct __align__(16) HydroSmem {
    double w[NR], m1[NR], m2[NR], p[NR];
    double b0[NR], bt[NR], bx[NR], by[NR];
    double Hn[NR], rho[NR], u[NR], v[NR], psi[NR];
    double gam[NR];     // gam of each loaded cell (a square root, taken once per pass)
    double lx[5][NLX];  // X slopes of (w, Hnpsi, u, v, rho), cells cx in [-1, BS], cy in [0, BS)
    double ly[5][NLX];  // Y slopes, cells cy in [-1, BS], cx in [0, BS)
    double fx[7][NFX];  // X-face fluxes: h(w, m1, m2, Hnpsi), g, p(m1), p(m2)
    double fy[7][NFX];  // Y-face fluxes
    double red[NT / 32];
};

__device__ __forceinline__ size_t plane(int slot, int nf, int f, int npl) {
    return ((size_t)slot * nf + f) * (size_t)npl;
}

// Stage formulas of HydraulicTimeStepper (src/TimeStepper.f90:371-515), operand order kept.
__device__ __forceinline__ void stage1(double q0[4], const double E[4], double I, double dt, double out[4]) {
    out[0] = q0[0] + dt * E[0];
    out[1] = (q0[1] + dt * E[1]) / (1.0 - dt * I);
    out[2] = (q0[2] + dt * E[2]) / (1.0 - dt * I);
    out[3] = q0[3] + dt * E[3];
}
__device__ __forceinline__ void stage23(int which, const double q0[4], const double qk[4], const double E[4], double I, double dt,
                                        double b00, double bt0, double b0k, double btk, double out[4]) {
    double hp_old = -bt0;
    hp_old = hp_old + (q0[0] - b00);
    double hp_new = -btk;
    hp_new = hp_new + (qk[0] - b0k);
    if (which == 2) {
        out[1] = 0.75 * q0[1] + 0.25 * (qk[1] + dt * E[1]) / (1.0 - dt * I);
        out[2] = 0.75 * q0[2] + 0.25 * (qk[2] + dt * E[2]) / (1.0 - dt * I);
        double w = bt0;
        w = w + 0.25 * hp_new;
        w = w + 0.75 * hp_old;
        w = w + 0.25 * dt * E[0];
        w = w + b00;
        out[0] = w;
        out[3] = 0.75 * q0[3] + 0.25 * (qk[3] + dt * E[3]);
    } else {
        const double third = 1.0 / 3.0, twothird = 2.0 / 3.0;
        out[1] = third * q0[1] + twothird * (qk[1] + dt * E[1]) / (1.0 - dt * I);
        out[2] = third * q0[2] + twothird * (qk[2] + dt * E[2]) / (1.0 - dt * I);
        double w = bt0;
        w = w + third * hp_old;
        w = w + twothird * hp_new;
        w = w + twothird * dt * E[0];
        w = w + b00;
        out[0] = w;
        out[3] = third * q0[3] + twothird * (qk[3] + dt * E[3]);
    }
}

// Desingularised variables (src/HydraulicRHS.f90:762-878) for one cell.
__device__ __forceinline__ void desing(const DevParams& P, double w, double m1, double m2, double pp, double b0, double bt,
                                       double gam, double& Hn, double& psi, double& rho, double& u, double& v) {
    Hn = compute_hn(w, b0, bt, gam);
    if (Hn < 0.0) Hn = 0.0;
    double Hnpsi = pp;
    if (Hnpsi < 0.0) Hnpsi = 0.0;
    double e2 = P.hThr * P.hThr;
    psi = mn(2.0 * Hn * Hnpsi / (Hn * Hn + mx(Hn * Hn, e2)), P.maxPack);
    rho = density(P, psi);
    u = 2.0 * Hn * m1 / (Hn * Hn + mx(Hn * Hn, e2)) / rho;
    v = 2.0 * Hn * m2 / (Hn * Hn + mx(Hn * Hn, e2)) / rho;
}

// Flux-source rates of ExplicitSourceTerms (src/Equations.f90:500-590) at cell centre
// (x, y): s1 = sum of Q / (NumCellsInSrc dx dy), s3 = the same for psi Q.
__device__ __forceinline__ void flux_source_rates(const DevParams& P, const DevSource* src, double t, double tg, double x,
                                                  double y, double& s1, double& s3) {
    for (int J = 0; J < P.nSources; ++J) {
        const DevSource& S = src[J];
        double Qf = 0.0, psiQf = 0.0;
        if (((x - S.x) * (x - S.x) + (y - S.y) * (y - S.y)) < S.R * S.R) {
            int n = S.n;
            if (n == 1) {
                if (!(t < S.time[0] || (t == S.time[0] && tg < t))) {
                    Qf = S.flux[0];
                    psiQf = S.psi[0] * Qf;
                }
            } else {
                if (!(t < S.time[0] || t > S.time[n - 1] || (t == S.time[0] && tg < t) || (t == S.time[n - 1] && tg == t))) {
                    for (int K = 1; K < n; ++K) {
                        if ((t >= S.time[K - 1]) && (t <= S.time[K])) {
                            double Qa = S.flux[K - 1], psia = S.psi[K - 1], ta = S.time[K - 1];
                            double Qb = S.flux[K], psib = S.psi[K], tb = S.time[K];
                            Qf = Qa + (Qb - Qa) * (t - ta) / (tb - ta);
                            double psif = psia + (psib - psia) * (t - ta) / (tb - ta);
                            psiQf = psif * Qf;
                        }
                    }
                }
            }
        }
        // A cell outside the source adds +0 either way; skip its divides.
        if (Qf != 0.0 || psiQf != 0.0) {
            double ncs = (double)S.ncells;
            Qf = Qf / ncs / P.dx / P.dy;
            psiQf = psiQf / ncs / P.dx / P.dy;
        }
        s1 = s1 + Qf;
        s3 = s3 + psiQf;
    }
}

// Flux-source and gravity terms of ExplicitSourceTerms (src/Equations.f90:456-620).
__device__ __forceinline__ void explicit_sources(const DevParams& P, bool has_src, double t, double tg, double x, double y,
                                                 double w, double b0, double bt, double rho, double dbdx, double dbdy,
                                                 double gam, double ste[4]) {
    double Qt = 0.0, psiQt = 0.0;
    if (has_src && P.nSources >= 1) {
        double s1 = 0.0, s3 = 0.0;
        flux_source_rates(P, cSrc, t, tg, x, y, s1, s3);
        Qt = Qt + s1;
        psiQt = psiQt + s3;
    }
    ste[0] = 0.0 + Qt / (gam * gam);
    ste[3] = 0.0 + psiQt / gam;
    double hp_o_gam = -bt;
    hp_o_gam = hp_o_gam + (w - b0);
    hp_o_gam = hp_o_gam / gam;
    ste[1] = 0.0 - P.g * rho * hp_o_gam * dbdx;
    ste[2] = 0.0 - P.g * rho * hp_o_gam * dbdy;
}

// One side of a face: the reconstructed state the flux formulas read.
struct Side {
    double w, p, u, v, rho, du, dv;  // du/dv: normal slopes of u and v (diffusion)
};

// Central-upwind fluxes at one face (CalculateFluxes body, src/HydraulicRHS.f90:949-1064
// for x, :1075-1180 for y).  'xdir' selects the normal velocity and tangential slope.
__device__ __forceinline__ void face_flux(const DevParams& P, bool xdir, const Side& Pl, const Side& Mi, double b0f, double btf,
                                          double dbxf, double dbyf, double gamL, double gamR, double h, double out[7],
                                          double& cfl) {
    double gamf = gam_of(P.geo, dbxf, dbyf);
    double HnP = compute_hn(Pl.w, b0f, btf, gamf);
    double HnM = compute_hn(Mi.w, b0f, btf, gamf);
    double unP = xdir ? Pl.u : Pl.v, unM = xdir ? Mi.u : Mi.v;
    double bt_ = xdir ? dbyf : dbxf;
    // Wave speeds u +- sqrt(g Hn (1 + b_t^2) / gam^3), Hn clamped at 0 (src/Equations.f90:249-381).
    double hP = HnP <= 0.0 ? 0.0 : HnP, hM = HnM <= 0.0 ? 0.0 : HnM;
    double cP, cM;
    if (P.geo) {
        cP = sqrt(P.g * hP * (1.0 + bt_ * bt_) / (gamf * gamf * gamf));
        cM = sqrt(P.g * hM * (1.0 + bt_ * bt_) / (gamf * gamf * gamf));
    } else {
        cP = sqrt(P.g * hP);
        cM = sqrt(P.g * hM);
    }
    double wsP = unP + cP, wsM = unM + cM;
    double aPos = (wsP > wsM) ? wsP : wsM;
    if (aPos < 0.0) aPos = 0.0;
    wsP = unP - cP;
    wsM = unM - cM;
    double aNeg = (wsP < wsM) ? wsP : wsM;
    if (aNeg > 0.0) aNeg = 0.0;
    if (aPos > kEPS) {
        double gr = mn(gamL / gamf, 1.0);
        cfl = mn(gr * gr * h / aPos, cfl);
    }
    if (fabs(aNeg) > kEPS) {
        double gr = mn(gamR / gamf, 1.0);
        cfl = mn(gr * gr * h / fabs(aNeg), cfl);
    }
    double dif = aPos - aNeg;
    if (dif < 1e-10) {
#pragma unroll
        for (int k = 0; k < 7; ++k) out[k] = 0.0;
        return;
    }
    // Face momenta rho*Hn*u / rho*Hn*v (src/HydraulicRHS.f90:521-551).
    double m1P = Pl.rho * HnP * Pl.u, m1M = Mi.rho * HnM * Mi.u;
    double m2P = Pl.rho * HnP * Pl.v, m2M = Mi.rho * HnM * Mi.v;
    // Convection fluxes (src/Equations.f90:53-104).
    double cwP = HnP * unP * gamf, cwM = HnM * unM * gamf;
    double cpP = Pl.p * unP * gamf, cpM = Mi.p * unM * gamf;
    double c1P = m1P * unP, c1M = m1M * unP;
    c1M = m1M * unM;
    double c2P = m2P * unP, c2M = m2M * unM;
    double hx;
    hx = HnP * gamf - HnM * gamf;
    hx = hx * aPos * aNeg;
    hx = hx + (aPos * cwM - aNeg * cwP);
    out[0] = hx / dif;
    hx = Pl.p * gamf - Mi.p * gamf;
    hx = hx * aPos * aNeg;
    hx = hx + (aPos * cpM - aNeg * cpP);
    out[3] = hx / dif;
    hx = m1P - m1M;
    hx = hx * aPos * aNeg;
    hx = hx + (aPos * c1M - aNeg * c1P);
    out[1] = hx / dif;
    hx = m2P - m2M;
    hx = hx * aPos * aNeg;
    hx = hx + (aPos * c2M - aNeg * c2P);
    out[2] = hx / dif;
    // Hydrostatic flux 0.5 g rho hp^2, identical in both momentum rows (src/Equations.f90:109-171).
    double hpP = -btf;
    hpP = hpP + (Pl.w - b0f);
    double hpM = -btf;
    hpM = hpM + (Mi.w - b0f);
    double GP = 0.5 * P.g * Pl.rho * hpP * hpP, GM = 0.5 * P.g * Mi.rho * hpM * hpM;
    out[4] = (aPos * GM - aNeg * GP) / dif;
    // Eddy-viscosity fluxes (src/Equations.f90:176-245).
    double dP1 = 0.0, dP2 = 0.0, dM1 = 0.0, dM2 = 0.0;
    if (!(HnP < 0.0)) {
        dP1 = P.nu * Pl.rho * HnP * Pl.du;
        dP2 = P.nu * Pl.rho * HnP * Pl.dv;
    }
    if (!(HnM < 0.0)) {
        dM1 = P.nu * Mi.rho * HnM * Mi.du;
        dM2 = P.nu * Mi.rho * HnM * Mi.dv;
    }
    out[5] = 0.5 * (dP1 + dM1);
    out[6] = 0.5 * (dP2 + dM2);
}

// ComputeAdvisedTimeStep (src/HydraulicRHS.f90:141-174) before the substep-1 factor, with
// the host's operation order.
__device__ __forceinline__ double advised_m(const DevParams& P, unsigned long long bits, int partial) {
    double umin = __longlong_as_double((long long)bits);
    if (partial) umin = mn(umin, P.maxdt);
    double m = mn(P.cfl * umin, P.diffusiveTimeScale);
    return mn(m, P.maxdt);
}

// The dt and times one pass uses.
struct StageTimes {
    double dt, t_rhs, t_max;
};

// Resolve a device-held dt (and the times derived from it exactly as the host derives
// them), then apply the stage gate: false when an earlier test of this step would have
// refined dt (TimeStepper.f90:393-404, :452-463 and the 10% test of :235-248), so the pass
// leaves every output untouched.  S stays in parameter space (constant indices only).
__device__ __forceinline__ bool stage_gate_open(const DevParams& P, const StepArgs& S, StageTimes& T) {
    T.dt = S.dt;
    T.t_rhs = S.t_rhs;
    T.t_max = S.t_max;
    if (S.dtp) {
        T.dt = *(volatile const double*)S.dtp;
        if (S.tmode == 1) T.t_rhs = S.t_grid + T.dt;
        else if (S.tmode == 2) T.t_rhs = S.t_grid + 0.5 * T.dt;
        T.t_max = S.t_grid + T.dt;
    }
    if (S.gate_flag && *(volatile const int*)S.gate_flag != 0) return false;
#pragma unroll
    for (int g = 0; g < 3; ++g) {
        if (g < S.ngate) {
            double m = advised_m(P, *(volatile const unsigned long long*)S.gate[g], S.partial);
            if (S.gate_s1[g]) m = 0.9 * m;
            if (m < T.dt) return false;
        }
    }
    return true;
}

// The gate and times are the same for every thread of a launch; lane 0 of each warp
// evaluates them (FP64 work, 1/64 of the FP32 rate on this GPU) and the warp takes them
// from it.  Every lane of the warp must call this.
__device__ __forceinline__ bool stage_gate_open_warp(const DevParams& P, const StepArgs& S, StageTimes& T) {
    int open = 0;
    if ((threadIdx.x & 31) == 0) open = stage_gate_open(P, S, T) ? 1 : 0;
    open = __shfl_sync(0xffffffffu, open, 0);
    T.dt = __shfl_sync(0xffffffffu, T.dt, 0);
    T.t_rhs = __shfl_sync(0xffffffffu, T.t_rhs, 0);
    T.t_max = __shfl_sync(0xffffffffu, T.t_max, 0);
    return open != 0;
}

// The first dt of a step on the device: IntegrateTo's min(advised dt of the RHS at t,
// the distance to the next flux knot) (src/TimeStepper.f90:151-183), from the CFL word of
// the RHS pass; cap is the host's (tmax - t) or (tmax - t)/2.
__global__ void k_dt(const unsigned long long* __restrict__ cfl, int partial, double cap, double* dtp) {
    kg_dep_wait();
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double adv = 0.9 * advised_m(cP, *cfl, partial);
        *dtp = mn(adv, cap);
    }
}

cudaError_t launch_dt(const unsigned long long* cfl, int partial, double cap, double* dtp, cudaStream_t st) {
    KG_TRY_LAUNCH(kg_launch(k_dt, 1, 32, 0, st, cfl, partial, cap, dtp));
    return cudaGetLastError();
}

__global__ void __launch_bounds__(NT) k_hydro(DevArrays A, const BlockDesc* __restrict__ blocks, const StepArgs S) {
    kg_dep_wait();
    StageTimes Tm;
    if (!stage_gate_open_warp(cP, S, Tm)) return;
    extern __shared__ __align__(16) unsigned char smraw[];
    HydroSmem& sm = *reinterpret_cast<HydroSmem*>(smraw);
    const DevParams& P = cP;
    const BlockDesc bd = blocks[blockIdx.x];
    const int nX = P.nX, nY = P.nY, SC = nX * nY, SFX = (nX + 1) * nY, SFY = nX * (nY + 1);
    const int slot = bd.slot;
    const int bx = min(BS, nX - bd.x0), by = min(BS, nY - bd.y0);
    const int tid = threadIdx.x;
    const int nbW = A.nbr[slot * 8 + NB_W], nbE = A.nbr[slot * 8 + NB_E];
    const int nbN = A.nbr[slot * 8 + NB_N], nbS = A.nbr[slot * 8 + NB_S];
    const double* __restrict__ Qin = (S.mode == MODE_RHS0 || S.mode == MODE_S1) ? A.Q[S.q_in]
                                   : (S.mode == MODE_S2)                        ? A.Q[S.q_s1]
                                                                                : A.Q[S.q_s2];
    const double* __restrict__ CT = A.CT[S.topo];
    const double* __restrict__ FX = A.FX[S.topo];
    const double* __restrict__ FY = A.FY[S.topo];

    // ---- A: load the cross-shaped region and desingularise ----
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
        double b0 = CT[plane(s, 4, 0, SC) + c], bt = CT[plane(s, 4, 1, SC) + c];
        double dbx = CT[plane(s, 4, 2, SC) + c], dby = CT[plane(s, 4, 3, SC) + c];
        sm.b0[r] = b0; sm.bt[r] = bt; sm.bx[r] = dbx; sm.by[r] = dby;
        const double gam = gam_of(P.geo, dbx, dby);
        sm.gam[r] = gam;
        if (A.kind[s] == SLOT_GHOST) {
            sm.w[r] = A.G9[plane(s, 9, 0, SC) + c];
            sm.m1[r] = A.G9[plane(s, 9, 1, SC) + c];
            sm.m2[r] = A.G9[plane(s, 9, 2, SC) + c];
            sm.p[r] = A.G9[plane(s, 9, 3, SC) + c];
            sm.Hn[r] = A.G9[plane(s, 9, 4, SC) + c];
            sm.u[r] = A.G9[plane(s, 9, 5, SC) + c];
            sm.v[r] = A.G9[plane(s, 9, 6, SC) + c];
            sm.psi[r] = A.G9[plane(s, 9, 7, SC) + c];
            sm.rho[r] = A.G9[plane(s, 9, 8, SC) + c];
            continue;
        }
        double q[4];
        if (S.mode == MODE_S1) {
            double q0[4], E[4];
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                q0[f] = Qin[plane(s, 4, f, SC) + c];
                E[f] = A.E[S.e_set][plane(s, 4, f, SC) + c];
            }
            stage1(q0, E, A.I[S.e_set][plane(s, 1, 0, SC) + c], Tm.dt, q);
        } else {
#pragma unroll
            for (int f = 0; f < 4; ++f) q[f] = Qin[plane(s, 4, f, SC) + c];
        }
        sm.w[r] = q[0]; sm.m1[r] = q[1]; sm.m2[r] = q[2]; sm.p[r] = q[3];
        double Hn, psi, rho, u, v;
        desing(P, q[0], q[1], q[2], q[3], b0, bt, gam, Hn, psi, rho, u, v);
        sm.Hn[r] = Hn; sm.psi[r] = psi; sm.rho[r] = rho; sm.u[r] = u; sm.v[r] = v;
    }
    __syncthreads();

    // ---- B: limited slopes ----
    const int lim = P.limiter;
    for (int kk = tid; kk < (bx + 2) * by + (by + 2) * bx; kk += NT) {
        if (kk < (bx + 2) * by) {
            const int k = kk;
            int cx = k % (bx + 2) - 1, cy = k / (bx + 2);
            int r = (cy + 2) * RG + (cx + 2);
            int li = cy * (BS + 2) + (cx + 1);
            bool ghW = (cx < 0 && bd.x0 == 0 && A.kind[nbW] == SLOT_GHOST);
            bool ghE = (cx >= bx && bd.x0 + bx == nX && A.kind[nbE] == SLOT_GHOST);
            if (ghW || ghE) {
                int gs = ghW ? nbW : nbE;
                sm.lx[0][li] = A.GE[plane(gs, GE_COUNT, ghW ? GE_LXN : GE_LX1, A.nE) + bd.y0 + cy];
                sm.lx[1][li] = 0.0; sm.lx[2][li] = 0.0; sm.lx[3][li] = 0.0; sm.lx[4][li] = 0.0;
            } else {
                sm.lx[0][li] = P.dxR * limiter(lim, sm.w[r + 1] - sm.w[r], sm.w[r] - sm.w[r - 1]);
                sm.lx[1][li] = P.dxR * limiter(lim, sm.p[r + 1] - sm.p[r], sm.p[r] - sm.p[r - 1]);
                sm.lx[2][li] = P.dxR * limiter(lim, sm.u[r + 1] - sm.u[r], sm.u[r] - sm.u[r - 1]);
                sm.lx[3][li] = P.dxR * limiter(lim, sm.v[r + 1] - sm.v[r], sm.v[r] - sm.v[r - 1]);
                sm.lx[4][li] = P.dxR * limiter(lim, sm.rho[r + 1] - sm.rho[r], sm.rho[r] - sm.rho[r - 1]);
            }
        } else {
            const int k = kk - ((bx + 2) * by);
            int cx = k % bx, cy = k / bx - 1;
            int r = (cy + 2) * RG + (cx + 2);
            int li = (cy + 1) * BS + cx;
            bool ghS = (cy < 0 && bd.y0 == 0 && A.kind[nbS] == SLOT_GHOST);
            bool ghN = (cy >= by && bd.y0 + by == nY && A.kind[nbN] == SLOT_GHOST);
            if (ghS || ghN) {
                int gs = ghS ? nbS : nbN;
                sm.ly[0][li] = A.GE[plane(gs, GE_COUNT, ghS ? GE_LYN : GE_LY1, A.nE) + bd.x0 + cx];
                sm.ly[1][li] = 0.0; sm.ly[2][li] = 0.0; sm.ly[3][li] = 0.0; sm.ly[4][li] = 0.0;
            } else {
                sm.ly[0][li] = P.dyR * limiter(lim, sm.w[r + RG] - sm.w[r], sm.w[r] - sm.w[r - RG]);
                sm.ly[1][li] = P.dyR * limiter(lim, sm.p[r + RG] - sm.p[r], sm.p[r] - sm.p[r - RG]);
                sm.ly[2][li] = P.dyR * limiter(lim, sm.u[r + RG] - sm.u[r], sm.u[r] - sm.u[r - RG]);
                sm.ly[3][li] = P.dyR * limiter(lim, sm.v[r + RG] - sm.v[r], sm.v[r] - sm.v[r - RG]);
                sm.ly[4][li] = P.dyR * limiter(lim, sm.rho[r + RG] - sm.rho[r], sm.rho[r] - sm.rho[r - RG]);
            }
        }
    }
    __syncthreads();

    // ---- C: face states, corrections, fluxes, CFL ----
    double cfl = 1.7976931348623157e308;
    const double hdx = 0.5, dx = P.dx, dy = P.dy;
    for (int kk = tid; kk < (bx + 1) * by + (by + 1) * bx; kk += NT) {
        if (kk < (bx + 1) * by) {
            const int k = kk;
            int fx = k % (bx + 1), cy = k / (bx + 1);
            int fi = bd.x0 + fx, j = bd.y0 + cy;
            int rL = (cy + 2) * RG + (fx + 1), rR = rL + 1;
            int liL = cy * (BS + 2) + fx, liR = liL + 1;
            Side L, R;
            // Left state: the right-face reconstruction of cell fx-1.
            double sw = sm.lx[0][liL], sp = sm.lx[1][liL];
            L.w = sm.w[rL] + sw * hdx * dx;
            L.p = sm.p[rL] + sp * hdx * dx;
            L.u = sm.u[rL] + sm.lx[2][liL] * hdx * dx;
            L.v = sm.v[rL] + sm.lx[3][liL] * hdx * dx;
            L.rho = sm.rho[rL] + sm.lx[4][liL] * hdx * dx;
            L.du = sm.lx[2][liL];
            L.dv = sm.lx[3][liL];
            if (fi == 0) {
                const double* fxs = FX + plane(nbW, 5, 4, SFX);
                double bl = fxs[j * (nX + 1) + nX - 1], br = fxs[j * (nX + 1) + nX];
                if (A.kind[nbW] == SLOT_GHOST) {
                    const double* ge = A.GE + plane(nbW, GE_COUNT, 0, A.nE);
                    if (ge[GE_MXN1 * A.nE + j] < br || ge[GE_PXN * A.nE + j] < bl) L.w = sm.w[rL] + 0.5 * (br - bl);
                } else {
                    double wl = sm.w[rL] - sw * hdx * dx;
                    if (L.w < br || wl < bl) L.w = sm.w[rL] + 0.5 * (br - bl);
                }
                if (L.p < 0.0) L.p = sm.p[rL];
            } else {
                const double* fxs = FX + plane(slot, 5, 4, SFX);
                double bl = fxs[j * (nX + 1) + fi - 1], br = fxs[j * (nX + 1) + fi];
                double wl = sm.w[rL] - sw * hdx * dx, pl = sm.p[rL] - sp * hdx * dx;
                if (L.w < br || wl < bl) L.w = sm.w[rL] + 0.5 * (br - bl);
                if (L.p < 0.0 || pl < 0.0) L.p = sm.p[rL];
            }
            // Right state: the left-face reconstruction of cell fx.
            sw = sm.lx[0][liR];
            sp = sm.lx[1][liR];
            R.w = sm.w[rR] - sw * hdx * dx;
            R.p = sm.p[rR] - sp * hdx * dx;
            R.u = sm.u[rR] - sm.lx[2][liR] * hdx * dx;
            R.v = sm.v[rR] - sm.lx[3][liR] * hdx * dx;
            R.rho = sm.rho[rR] - sm.lx[4][liR] * hdx * dx;
            R.du = sm.lx[2][liR];
            R.dv = sm.lx[3][liR];
            if (fi == nX) {
                const double* fxs = FX + plane(nbE, 5, 4, SFX);
                double bl = fxs[j * (nX + 1) + 0], br = fxs[j * (nX + 1) + 1];
                if (A.kind[nbE] == SLOT_GHOST) {
                    const double* ge = A.GE + plane(nbE, GE_COUNT, 0, A.nE);
                    if (ge[GE_MX2 * A.nE + j] < br || ge[GE_PX1 * A.nE + j] < bl) R.w = sm.w[rR] + 0.5 * (bl - br);
                } else {
                    double wr = sm.w[rR] + sw * hdx * dx;
                    if (wr < br || R.w < bl) R.w = sm.w[rR] + 0.5 * (bl - br);
                }
                if (R.p < 0.0) R.p = sm.p[rR];
            } else {
                const double* fxs = FX + plane(slot, 5, 4, SFX);
                double bl = fxs[j * (nX + 1) + fi], br = fxs[j * (nX + 1) + fi + 1];
                double wr = sm.w[rR] + sw * hdx * dx, pr = sm.p[rR] + sp * hdx * dx;
                if (wr < br || R.w < bl) R.w = sm.w[rR] + 0.5 * (bl - br);
                if (pr < 0.0 || R.p < 0.0) R.p = sm.p[rR];
            }
            size_t fo = (size_t)slot * 5 * SFX + (size_t)j * (nX + 1) + fi;
            double b0f = FX[fo], btf = FX[fo + SFX], dbxf = FX[fo + 2 * (size_t)SFX], dbyf = FX[fo + 3 * (size_t)SFX];
            double gamL = sm.gam[rL], gamR = sm.gam[rR];
            double out[7];
            face_flux(P, true, R, L, b0f, btf, dbxf, dbyf, gamL, gamR, dx, out, cfl);
            int fo2 = cy * (BS + 1) + fx;
    #pragma unroll
            for (int q = 0; q < 7; ++q) sm.fx[q][fo2] = out[q];
        } else {
            const int k = kk - ((bx + 1) * by);
            int cx = k % bx, fy = k / bx;
            int fj = bd.y0 + fy, i = bd.x0 + cx;
            int rL = (fy + 1) * RG + (cx + 2), rR = rL + RG;
            int liL = fy * BS + cx, liR = liL + BS;
            Side L, R;
            double sw = sm.ly[0][liL], sp = sm.ly[1][liL];
            L.w = sm.w[rL] + sw * hdx * dy;
            L.p = sm.p[rL] + sp * hdx * dy;
            L.u = sm.u[rL] + sm.ly[2][liL] * hdx * dy;
            L.v = sm.v[rL] + sm.ly[3][liL] * hdx * dy;
            L.rho = sm.rho[rL] + sm.ly[4][liL] * hdx * dy;
            L.du = sm.ly[2][liL];
            L.dv = sm.ly[3][liL];
            if (fj == 0) {
                const double* fys = FY + plane(nbS, 5, 4, SFY);
                double bb = fys[(nY - 1) * nX + i], bt_ = fys[nY * nX + i];
                if (A.kind[nbS] == SLOT_GHOST) {
                    const double* ge = A.GE + plane(nbS, GE_COUNT, 0, A.nE);
                    if (ge[GE_MYN1 * A.nE + i] < bt_ || ge[GE_PYN * A.nE + i] < bb) L.w = sm.w[rL] + 0.5 * (bt_ - bb);
                } else {
                    double wb = sm.w[rL] - sw * hdx * dy;
                    if (L.w < bt_ || wb < bb) L.w = sm.w[rL] + 0.5 * (bt_ - bb);
                }
                if (L.p < 0.0) L.p = sm.p[rL];
            } else {
                const double* fys = FY + plane(slot, 5, 4, SFY);
                double bb = fys[(fj - 1) * nX + i], bt_ = fys[fj * nX + i];
                double wb = sm.w[rL] - sw * hdx * dy, pb = sm.p[rL] - sp * hdx * dy;
                if (L.w < bt_ || wb < bb) L.w = sm.w[rL] + 0.5 * (bt_ - bb);
                if (L.p < 0.0 || pb < 0.0) L.p = sm.p[rL];
            }
            sw = sm.ly[0][liR];
            sp = sm.ly[1][liR];
            R.w = sm.w[rR] - sw * hdx * dy;
            R.p = sm.p[rR] - sp * hdx * dy;
            R.u = sm.u[rR] - sm.ly[2][liR] * hdx * dy;
            R.v = sm.v[rR] - sm.ly[3][liR] * hdx * dy;
            R.rho = sm.rho[rR] - sm.ly[4][liR] * hdx * dy;
            R.du = sm.ly[2][liR];
            R.dv = sm.ly[3][liR];
            if (fj == nY) {
                const double* fys = FY + plane(nbN, 5, 4, SFY);
                double bb = fys[0 * nX + i], bt_ = fys[1 * nX + i];
                if (A.kind[nbN] == SLOT_GHOST) {
                    const double* ge = A.GE + plane(nbN, GE_COUNT, 0, A.nE);
                    if (ge[GE_MY2 * A.nE + i] < bt_ || ge[GE_PY1 * A.nE + i] < bb) R.w = sm.w[rR] + 0.5 * (bb - bt_);
                } else {
                    double wt = sm.w[rR] + sw * hdx * dy;
                    if (wt < bt_ || R.w < bb) R.w = sm.w[rR] + 0.5 * (bb - bt_);
                }
                if (R.p < 0.0) R.p = sm.p[rR];
            } else {
                const double* fys = FY + plane(slot, 5, 4, SFY);
                double bb = fys[fj * nX + i], bt_ = fys[(fj + 1) * nX + i];
                double wt = sm.w[rR] + sw * hdx * dy, pt = sm.p[rR] + sp * hdx * dy;
                if (wt < bt_ || R.w < bb) R.w = sm.w[rR] + 0.5 * (bb - bt_);
                if (pt < 0.0 || R.p < 0.0) R.p = sm.p[rR];
            }
            size_t fo = (size_t)slot * 5 * SFY + (size_t)fj * nX + i;
            double b0f = FY[fo], btf = FY[fo + SFY], dbxf = FY[fo + 2 * (size_t)SFY], dbyf = FY[fo + 3 * (size_t)SFY];
            double gamL = sm.gam[rL], gamR = sm.gam[rR];
            double out[7];
            face_flux(P, false, R, L, b0f, btf, dbxf, dbyf, gamL, gamR, dy, out, cfl);
            int fo2 = fy * BS + cx;
    #pragma unroll
            for (int q = 0; q < 7; ++q) sm.fy[q][fo2] = out[q];
        }
    }
    // CFL: warp then block min, one atomic per CTA (ordered bits of a positive double).
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cfl = mn(cfl, __shfl_xor_sync(0xffffffffu, cfl, o));
    if ((tid & 31) == 0) sm.red[tid >> 5] = cfl;
    __syncthreads();
    if (tid == 0) {
        double m = sm.red[0];
        for (int q = 1; q < NT / 32; ++q) m = mn(m, sm.red[q]);
        atomicMin(S.cfl_min, (unsigned long long)__double_as_longlong(m));
    }

    // ---- D: RHS assembly and stage update for the block's own cells ----
    if (tid < bx * by) {
        int cx = tid % bx, cy = tid / bx;
        int i = bd.x0 + cx, j = bd.y0 + cy, c = j * nX + i;
        int r = (cy + 2) * RG + (cx + 2);
        double b0 = sm.b0[r], bt = sm.bt[r], dbdx = sm.bx[r], dbdy = sm.by[r];
        double gam = sm.gam[r];
        double gXp1, gXp2, gYp1, gYp2;
        if (P.geo) {
            gXp1 = (1.0 + dbdy * dbdy) / gam;
            gXp2 = -dbdx * dbdy / gam;
            gYp1 = -dbdx * dbdy / gam;
            gYp2 = (1.0 + dbdx * dbdx) / gam;
        } else {
            gXp1 = 1.0; gXp2 = 0.0; gYp1 = 0.0; gYp2 = 1.0;
        }
        int xl = cy * (BS + 1) + cx, xr = xl + 1;
        int yb = cy * BS + cx, yt = yb + BS;
        double STF[4];
        STF[0] = (sm.fx[0][xl] - sm.fx[0][xr]) * P.dxR / (gam * gam) + (sm.fy[0][yb] - sm.fy[0][yt]) * P.dyR / (gam * gam);
        STF[3] = (sm.fx[3][xl] - sm.fx[3][xr]) * P.dxR / gam + (sm.fy[3][yb] - sm.fy[3][yt]) * P.dyR / gam;
        STF[1] = kahan3(sm.fx[1][xl] - sm.fx[1][xr], (sm.fx[4][xl] - sm.fx[4][xr]) * gXp1, sm.fx[5][xr] - sm.fx[5][xl]) * P.dxR;
        STF[1] = STF[1] + kahan3(sm.fy[1][yb] - sm.fy[1][yt], (sm.fy[4][yb] - sm.fy[4][yt]) * gYp1, sm.fy[5][yt] - sm.fy[5][yb]) * P.dyR;
        STF[2] = kahan3(sm.fx[2][xl] - sm.fx[2][xr], (sm.fx[4][xl] - sm.fx[4][xr]) * gXp2, sm.fx[6][xr] - sm.fx[6][xl]) * P.dxR;
        STF[2] = STF[2] + kahan3(sm.fy[2][yb] - sm.fy[2][yt], (sm.fy[4][yb] - sm.fy[4][yt]) * gYp2, sm.fy[6][yt] - sm.fy[6][yb]) * P.dyR;
        int gi = (bd.tile - 1) % P.nXtiles + 1, gj = (bd.tile - 1) / P.nXtiles + 1;
        double x = -0.5 * P.xSize + P.dx * ((gi - 1.0) * P.nX + ((i + 1) - 0.5));
        double y = -0.5 * P.ySize + P.dy * ((gj - 1.0) * P.nY + ((j + 1) - 0.5));
        double ste[4];
        explicit_sources(P, A.has_source[slot] != 0, Tm.t_rhs, S.t_grid, x, y, sm.w[r], b0, bt, sm.rho[r], dbdx, dbdy, gam, ste);
        double E[4];
#pragma unroll
        for (int f = 0; f < 4; ++f) E[f] = STF[f] + ste[f];
        Pt<double> pt{sm.Hn[r], sm.u[r], sm.v[r], sm.psi[r], sm.rho[r], bt, dbdx, dbdy, gam};
        double I = implicit_source(P, pt, drag(P, pt));
        double qk[4] = {sm.w[r], sm.m1[r], sm.m2[r], sm.p[r]};
        if (S.mode == MODE_RHS0) {
#pragma unroll
            for (int f = 0; f < 4; ++f) A.E[S.e_set][plane(slot, 4, f, SC) + c] = E[f];
            A.I[S.e_set][plane(slot, 1, 0, SC) + c] = I;
        } else if (S.mode == MODE_S1 || S.mode == MODE_S2) {
            const double* q0p = A.Q[S.q_in];
            double q0[4], out[4];
#pragma unroll
            for (int f = 0; f < 4; ++f) q0[f] = q0p[plane(slot, 4, f, SC) + c];
            stage23(S.mode == MODE_S1 ? 2 : 3, q0, qk, E, I, Tm.dt, b0, bt, b0, bt, out);
            double* dst = A.Q[S.mode == MODE_S1 ? S.q_s1 : S.q_s2];
#pragma unroll
            for (int f = 0; f < 4; ++f) dst[plane(slot, 4, f, SC) + c] = out[f];
        } else {
            double dt = Tm.dt;
            double m1 = (qk[1] - dt * dt * E[1] * I) / (1.0 + dt * dt * I * I);
            double m2 = (qk[2] - dt * dt * E[2] * I) / (1.0 + dt * dt * I * I);
            double* dst = A.Q[S.q_out];
            dst[plane(slot, 4, 0, SC) + c] = qk[0];
            dst[plane(slot, 4, 1, SC) + c] = m1;
            dst[plane(slot, 4, 2, SC) + c] = m2;
            dst[plane(slot, 4, 3, SC) + c] = qk[3];
            A.UV[plane(slot, 2, 0, SC) + c] = sm.u[r];
            A.UV[plane(slot, 2, 1, SC) + c] = sm.v[r];
            if (S.do_maxima) {
                // UpdateMaximum* on the state at the start of the step
                // (src/TimeStepper.f90:519-524, :1155-1303).
                const double* q0p = A.Q[S.q_tc];
                const double* ct0 = A.CT[S.topo_tc];
                double b0t = ct0[plane(slot, 4, 0, SC) + c], btt = ct0[plane(slot, 4, 1, SC) + c];
                double dbxt = ct0[plane(slot, 4, 2, SC) + c], dbyt = ct0[plane(slot, 4, 3, SC) + c];
                double gamt = gam_of(P.geo, dbxt, dbyt);
                double Hn, psi, rho, u, v;
                desing(P, q0p[plane(slot, 4, 0, SC) + c], q0p[plane(slot, 4, 1, SC) + c], q0p[plane(slot, 4, 2, SC) + c],
                       q0p[plane(slot, 4, 3, SC) + c], b0t, btt, gamt, Hn, psi, rho, u, v);
                bt = btt;
                dbdx = dbxt;
                dbdy = dbyt;
                double* M = A.MX + plane(slot, 11, 0, SC) + c;
                double tt = Tm.t_max;
                if (Hn > P.hThr) {
                    if (M[10 * (size_t)SC] == -1.0) M[10 * (size_t)SC] = tt;
                    if (Hn > M[0]) { M[0] = Hn; M[(size_t)SC] = tt; }
                }
                double spd = sqrt(modu2_of(P.geo, u, v, dbdx, dbdy));
                if ((spd > M[2 * (size_t)SC]) && (Hn > P.hThr)) { M[2 * (size_t)SC] = spd; M[3 * (size_t)SC] = tt; }
                if (bt < 0.0 && -bt > M[4 * (size_t)SC]) { M[4 * (size_t)SC] = -bt; M[5 * (size_t)SC] = tt; }
                if (bt > 0.0 && bt > M[6 * (size_t)SC]) { M[6 * (size_t)SC] = bt; M[7 * (size_t)SC] = tt; }
                if (Hn > P.hThr && psi > M[8 * (size_t)SC]) { M[8 * (size_t)SC] = psi; M[9 * (size_t)SC] = tt; }
            }
        }
    }
}

size_t hydro_smem_bytes() { return sizeof(HydroSmem); }

cudaError_t set_constants(const DevParams& p, const DevSource* src, int nsrc, cudaStream_t st) {
    cudaError_t e = cudaMemcpyToSymbolAsync(cP, &p, sizeof(DevParams), 0, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    // A copy from pageable host memory is staged before the call returns, so a local
    // source is safe.
    const DevParams32 p32 = params32(p);
    e = cudaMemcpyToSymbolAsync(cP32, &p32, sizeof(DevParams32), 0, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    if (nsrc > 0) e = cudaMemcpyToSymbolAsync(cSrc, src, sizeof(DevSource) * nsrc, 0, cudaMemcpyHostToDevice, st);
    return e;
}

cudaError_t launch_hydro(const DevArrays& A, const BlockDesc* blocks, int nblocks, const StepArgs& S, cudaStream_t st) {
    // the shared-memory opt-in is a per-device function attribute: set once per device
    static bool attr[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!attr[dev]) {
        e = cudaFuncSetAttribute(k_hydro, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(HydroSmem));
        if (e != cudaSuccess) return e;
        attr[dev] = true;
    }
    if (nblocks == 0) return cudaSuccess;
    KG_TRY_LAUNCH(kg_launch(k_hydro, nblocks, NT, sizeof(HydroSmem), st, A, blocks, S));
    return cudaGetLastError();
}

}  // namespace kg
