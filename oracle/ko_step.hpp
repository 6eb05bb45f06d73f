// ko_step.hpp -- TEST INFRASTRUCTURE (the oracle).  RHS assembly, the morphodynamic
// operator, redistribution, tile activation and the time stepper, restated from
// src/HydraulicRHS.f90:1190-1304, src/Equations.f90:456-620, src/MorphodynamicRHS.f90,
// src/Redistribute.f90, src/UpdateTiles.f90, src/TimeStepper.f90, src/SetSources.f90 and
// src/Output.f90:617-737.
#pragma once
#include "ko_grid.hpp"
#include <stdexcept>

namespace ko {

// ExplicitSourceTerms, src/Equations.f90:456-620; writes ste[0..3] (w, rhoHnu, rhoHnv, Hnpsi).
inline void ExplicitSourceTerms(const RunSet& rp, const Grid& g, double t, double x, double y, const double* uv,
                                bool tile_has_source, double* ste) {
    for (int k = 0; k < 4; ++k) ste[k] = 0.0;
    double Qt = 0.0, rhoQt = 0.0, psiQt = 0.0;
    int nSrc = rp.nSources();
    if (tile_has_source && nSrc >= 1) {
        std::vector<double> Qf(nSrc, 0.0), rhoQf(nSrc, 0.0), psiQf(nSrc, 0.0);
        for (int J = 0; J < nSrc; ++J) {
            const FluxSrc& S = rp.FluxSources[J];
            if (((x - S.x) * (x - S.x) + (y - S.y) * (y - S.y)) < S.Radius * S.Radius) {
                int n = S.nFluxSeries;
                if (n == 1) {
                    if (t < S.time[0] || (t == S.time[0] && g.t < t)) {
                        Qf[J] = 0.0; rhoQf[J] = 0.0; psiQf[J] = 0.0;
                    } else {
                        Qf[J] = S.flux[0];
                        double rho = Density(rp, S.psi[0]);
                        rhoQf[J] = rho * Qf[J];
                        psiQf[J] = S.psi[0] * Qf[J];
                    }
                } else {
                    if (t < S.time[0] || t > S.time[n - 1] || (t == S.time[0] && g.t < t) ||
                        (t == S.time[n - 1] && g.t == t)) {
                        Qf[J] = 0.0; rhoQf[J] = 0.0; psiQf[J] = 0.0;
                    } else {
                        for (int K = 1; K < n; ++K) {
                            if ((t >= S.time[K - 1]) && (t <= S.time[K])) {
                                double Qa = S.flux[K - 1], psia = S.psi[K - 1], ta = S.time[K - 1];
                                double Qb = S.flux[K], psib = S.psi[K], tb = S.time[K];
                                Qf[J] = Qa + (Qb - Qa) * (t - ta) / (tb - ta);
                                double psif = psia + (psib - psia) * (t - ta) / (tb - ta);
                                double rho = Density(rp, psif);
                                rhoQf[J] = rho * Qf[J];
                                psiQf[J] = psif * Qf[J];
                            }
                        }
                    }
                }
            }
            double ncs = (double)S.NumCellsInSrc;
            Qf[J] = Qf[J] / ncs / g.deltaX / g.deltaY;
            rhoQf[J] = rhoQf[J] / ncs / g.deltaX / g.deltaY;
            psiQf[J] = psiQf[J] / ncs / g.deltaX / g.deltaY;
        }
        double s1 = 0.0, s2 = 0.0, s3 = 0.0;
        for (int J = 0; J < nSrc; ++J) { s1 = s1 + Qf[J]; s2 = s2 + rhoQf[J]; s3 = s3 + psiQf[J]; }
        Qt = Qt + s1;
        rhoQt = rhoQt + s2;
        psiQt = psiQt + s3;
    }
    double gam = Gam(rp, uv);
    double dbdx = uv[idbdx - 1], dbdy = uv[idbdy - 1];
    ste[0] = ste[0] + Qt / (gam * gam);
    ste[3] = ste[3] + psiQt / gam;
    double hp_o_gam = -uv[ibt - 1];
    hp_o_gam = hp_o_gam + (uv[iw - 1] - uv[ib0 - 1]);
    hp_o_gam = hp_o_gam / gam;
    ste[1] = ste[1] - rp.g * uv[irho - 1] * hp_o_gam * dbdx;
    ste[2] = ste[2] - rp.g * uv[irho - 1] * hp_o_gam * dbdy;
}

// ConstructHydraulicRHS, src/HydraulicRHS.f90:1190-1271 (2D).
inline void ConstructHydraulicRHS(const RunSet& rp, Grid& g, Tiles& tiles, int tID, double t) {
    Tile& T = TL(tiles, tID);
    double dxR = g.deltaXRecip, dyR = g.deltaYRecip;
    double gXp[4] = {0, 0, 0, 0}, gYp[4] = {0, 0, 0, 0};
    double STF[4], STE[4];
    for (int i = 1; i <= rp.nXpertile; ++i)
        for (int j = 1; j <= rp.nYpertile; ++j) {
            const double* uv = T.u.col(i, j);
            double gam = Gam(rp, uv);
            double dbdx = uv[idbdx - 1], dbdy = uv[idbdy - 1];
            if (rp.geometric_factors) {
                gXp[1] = (1.0 + dbdy * dbdy) / gam;
                gXp[2] = -dbdx * dbdy / gam;
                gYp[1] = -dbdx * dbdy / gam;
                gYp[2] = (1.0 + dbdx * dbdx) / gam;
            } else {
                gXp[1] = 1.0; gXp[2] = 0.0; gYp[1] = 0.0; gYp[2] = 1.0;
            }
            for (int k = 0; k < 4; ++k) {
                int d = IFLUX[k];
                if (d == iw) {
                    STF[k] = (T.hXFlux(d, i, j) - T.hXFlux(d, i + 1, j)) * dxR / (gam * gam) +
                             (T.hYFlux(d, i, j) - T.hYFlux(d, i, j + 1)) * dyR / (gam * gam);
                } else if (d == iHnpsi) {
                    STF[k] = (T.hXFlux(d, i, j) - T.hXFlux(d, i + 1, j)) * dxR / gam +
                             (T.hYFlux(d, i, j) - T.hYFlux(d, i, j + 1)) * dyR / gam;
                } else {
                    double ax[3] = {T.hXFlux(d, i, j) - T.hXFlux(d, i + 1, j),
                                    (T.gXFlux(d, i, j) - T.gXFlux(d, i + 1, j)) * gXp[k],
                                    T.pXFlux(d, i + 1, j) - T.pXFlux(d, i, j)};
                    STF[k] = KahanSumL(ax) * dxR;
                    double ay[3] = {T.hYFlux(d, i, j) - T.hYFlux(d, i, j + 1),
                                    (T.gYFlux(d, i, j) - T.gYFlux(d, i, j + 1)) * gYp[k],
                                    T.pYFlux(d, i, j + 1) - T.pYFlux(d, i, j)};
                    STF[k] = STF[k] + KahanSumL(ay) * dyR;
                }
            }
            ExplicitSourceTerms(rp, g, t, T.x[i - 1], T.y[j - 1], uv, T.containsSource, STE);
            for (int k = 0; k < 4; ++k) T.ddtExplicit(k + 1, i, j) = STF[k] + STE[k];
            double Friction = DragClosure(rp, uv);
            double sti = ImplicitMomentumSource(rp, uv, Friction);
            T.ddtImplicit(1, i, j) = 0.0;
            T.ddtImplicit(2, i, j) = sti;
            T.ddtImplicit(3, i, j) = sti;
            T.ddtImplicit(4, i, j) = 0.0;
        }
}

// ComputeAdvisedTimeStep, src/HydraulicRHS.f90:141-174.
inline double ComputeAdvisedTimeStep(const RunSet& rp, Grid& g, int substep, const std::vector<double>& unitCFL) {
    double mn = HUGE_;
    for (double v : unitCFL) mn = std::min(mn, v);
    double maxTimeStep = std::min(rp.cfl * mn, rp.diffusiveTimeScale);
    maxTimeStep = std::min(maxTimeStep, rp.maxdt);
    if (substep == 1) {
        double a = 0.9 * maxTimeStep;
        g.dt = a;
        return a;
    }
    return maxTimeStep;
}

// CalculateHydraulicRHS, src/HydraulicRHS.f90:64-136.
inline double CalculateHydraulicRHS(const RunSet& rp, Grid& g, Tiles& ws, double t, int substep) {
    std::vector<double> unitCFL((size_t)g.nTiles, rp.maxdt);
    const std::vector<int> act = g.activeTiles;
    for (int id : act) CalculateLimitedDerivs(rp, g, IFLUX, 4, ws, id);
    for (int id : act) Reconstruct(rp, g, IFLUX, 4, true, ws, id);
    for (int id : act) CorrectSlopes(rp, g, ws, id);
    for (int id : act) ComputeDesingularisedVariables(rp, ws, id, true);
    for (int id : act) CalculateLimitedDerivs(rp, g, IDESING, 5, ws, id);
    for (int id : act) Reconstruct(rp, g, IDESING, 5, false, ws, id);
    for (int id : act) CalculateFluxes(rp, g, ws, id, unitCFL[(size_t)id - 1]);
    double adv = ComputeAdvisedTimeStep(rp, g, substep, unitCFL);
    for (int id : act) ConstructHydraulicRHS(rp, g, ws, id, t);
    return adv;
}

// ---------------------------------------------------------------- MorphodynamicRHS.f90
// BtSourceTerm, :154-305 (2D).  The two pre-added Kahan entries (:210 west boundary,
// :266 NE corner) are kept exactly as written.
inline void BtSourceTerm(const RunSet& rp, Grid& g, Tiles& tiles) {
    int nX = rp.nXpertile, nY = rp.nYpertile;
    double psib = 1.0 - rp.p.BedPorosity;
    for (int tID : g.activeTiles) {
        Tile& T = TL(tiles, tID);
        for (int i = 2; i <= nX; ++i)
            for (int j = 2; j <= nY; ++j) {
                double ax[4] = {T.u(idbdx, i - 1, j - 1), T.u(idbdx, i - 1, j), T.u(idbdx, i, j - 1), T.u(idbdx, i, j)};
                double ay[4] = {T.u(idbdy, i - 1, j - 1), T.u(idbdy, i - 1, j), T.u(idbdy, i, j - 1), T.u(idbdy, i, j)};
                double gam = Gam_gradin(rp, 0.25 * KahanSumL(ax), 0.25 * KahanSumL(ay));
                double ae[4] = {T.EminusD(i - 1, j - 1), T.EminusD(i - 1, j), T.EminusD(i, j - 1), T.EminusD(i, j)};
                T.ddtExplicitBt(i, j) = -0.25 * gam / psib * KahanSumL(ae);
            }
        int ttW = T.West(), ttE = T.East(), ttS = T.South(), ttN = T.North();
        Tile &W = TL(tiles, ttW), &E = TL(tiles, ttE), &S = TL(tiles, ttS), &N = TL(tiles, ttN);
        // The diagonal tiles: on periodic domains one may never have been allocated (no
        // corner ghosts, src/UpdateTiles.f90:415-418), where the reference reads unallocated
        // data; it contributes zero here, as on the GPU.
        auto du = [](const Tile& X, int f, int i, int j) { return X.u.allocated() ? X.u(f, i, j) : 0.0; };
        auto de = [](const Tile& X, int i, int j) { return X.EminusD.allocated() ? X.EminusD(i, j) : 0.0; };
        Tile& SW = TL(tiles, W.South());
        Tile& SE = TL(tiles, E.South());
        Tile& NW = TL(tiles, W.North());
        Tile& NE = TL(tiles, E.North());
        for (int j = 2; j <= nY; ++j) {
            {
                double ax[4] = {W.u(idbdx, nX, j - 1), W.u(idbdx, nX, j), T.u(idbdx, 1, j - 1), T.u(idbdx, 1, j)};
                double ay[4] = {W.u(idbdy, nX, j - 1), W.u(idbdy, nX, j), T.u(idbdy, 1, j - 1), T.u(idbdy, 1, j)};
                double gam = Gam_gradin(rp, 0.25 * KahanSumL(ax), 0.25 * KahanSumL(ay));
                double ae[3] = {W.EminusD(nX, j - 1), W.EminusD(nX, j), T.EminusD(1, j - 1) + T.EminusD(1, j)};
                T.ddtExplicitBt(1, j) = -0.25 * gam / psib * KahanSumL(ae);
            }
            {
                double ax[4] = {T.u(idbdx, nX, j - 1), T.u(idbdx, nX, j), E.u(idbdx, 1, j - 1), E.u(idbdx, 1, j)};
                double ay[4] = {T.u(idbdy, nX, j - 1), T.u(idbdy, nX, j), E.u(idbdy, 1, j - 1), E.u(idbdy, 1, j)};
                double gam = Gam_gradin(rp, 0.25 * KahanSumL(ax), 0.25 * KahanSumL(ay));
                double ae[4] = {T.EminusD(nX, j - 1), T.EminusD(nX, j), E.EminusD(1, j - 1), E.EminusD(1, j)};
                T.ddtExplicitBt(nX + 1, j) = -0.25 * gam / psib * KahanSumL(ae);
            }
        }
        for (int i = 2; i <= nX; ++i) {
            {
                double ax[4] = {T.u(idbdx, i - 1, nY), N.u(idbdx, i - 1, 1), T.u(idbdx, i, nY), N.u(idbdx, i, 1)};
                double ay[4] = {T.u(idbdy, i - 1, nY), N.u(idbdy, i - 1, 1), T.u(idbdy, i, nY), N.u(idbdy, i, 1)};
                double gam = Gam_gradin(rp, 0.25 * KahanSumL(ax), 0.25 * KahanSumL(ay));
                double ae[4] = {T.EminusD(i - 1, nY), N.EminusD(i - 1, 1), T.EminusD(i, nY), N.EminusD(i, 1)};
                T.ddtExplicitBt(i, nY + 1) = -0.25 * gam / psib * KahanSumL(ae);
            }
            {
                double ax[4] = {S.u(idbdx, i - 1, nY), T.u(idbdx, i - 1, 1), S.u(idbdx, i, nY), T.u(idbdx, i, 1)};
                double ay[4] = {S.u(idbdy, i - 1, nY), T.u(idbdy, i - 1, 1), S.u(idbdy, i, nY), T.u(idbdy, i, 1)};
                double gam = Gam_gradin(rp, 0.25 * KahanSumL(ax), 0.25 * KahanSumL(ay));
                double ae[4] = {S.EminusD(i - 1, nY), T.EminusD(i - 1, 1), S.EminusD(i, nY), T.EminusD(i, 1)};
                T.ddtExplicitBt(i, 1) = -0.25 * gam / psib * KahanSumL(ae);
            }
        }
        {  // SW
            double ax[4] = {du(SW, idbdx, nX, nY), W.u(idbdx, nX, 1), S.u(idbdx, 1, nY), T.u(idbdx, 1, 1)};
            double ay[4] = {du(SW, idbdy, nX, nY), W.u(idbdy, nX, 1), S.u(idbdy, 1, nY), T.u(idbdy, 1, 1)};
            double gam = Gam_gradin(rp, 0.25 * KahanSumL(ax), 0.25 * KahanSumL(ay));
            double ae[4] = {de(SW, nX, nY), W.EminusD(nX, 1), S.EminusD(1, nY), T.EminusD(1, 1)};
            T.ddtExplicitBt(1, 1) = -0.25 * gam / psib * KahanSumL(ae);
        }
        {  // SE
            double ax[4] = {S.u(idbdx, nX, nY), T.u(idbdx, nX, 1), du(SE, idbdx, 1, nY), E.u(idbdx, 1, 1)};
            double ay[4] = {S.u(idbdy, nX, nY), T.u(idbdy, nX, 1), du(SE, idbdy, 1, nY), E.u(idbdy, 1, 1)};
            double gam = Gam_gradin(rp, 0.25 * KahanSumL(ax), 0.25 * KahanSumL(ay));
            double ae[4] = {S.EminusD(nX, nY), T.EminusD(nX, 1), de(SE, 1, nY), E.EminusD(1, 1)};
            T.ddtExplicitBt(nX + 1, 1) = -0.25 * gam / psib * KahanSumL(ae);
        }
        {  // NW
            double ax[4] = {W.u(idbdx, nX, nY), du(NW, idbdx, nX, 1), T.u(idbdx, 1, nY), N.u(idbdx, 1, 1)};
            double ay[4] = {W.u(idbdy, nX, nY), du(NW, idbdy, nX, 1), T.u(idbdy, 1, nY), N.u(idbdy, 1, 1)};
            double gam = Gam_gradin(rp, 0.25 * KahanSumL(ax), 0.25 * KahanSumL(ay));
            double ae[4] = {W.EminusD(nX, nY), de(NW, nX, 1), T.EminusD(1, nY), N.EminusD(1, 1)};
            T.ddtExplicitBt(1, nY + 1) = -0.25 * gam / psib * KahanSumL(ae);
        }
        {  // NE
            double ax[3] = {T.u(idbdx, nX, nY), N.u(idbdx, nX, 1), E.u(idbdx, 1, nY) + du(NE, idbdx, 1, 1)};
            double ay[4] = {T.u(idbdy, nX, nY), N.u(idbdy, nX, 1), E.u(idbdy, 1, nY), du(NE, idbdy, 1, 1)};
            double gam = Gam_gradin(rp, 0.25 * KahanSumL(ax), 0.25 * KahanSumL(ay));
            double ae[4] = {T.EminusD(nX, nY), N.EminusD(nX, 1), E.EminusD(1, nY), de(NE, 1, 1)};
            T.ddtExplicitBt(nX + 1, nY + 1) = -0.25 * gam / psib * KahanSumL(ae);
        }
    }
}

// CalculateMorphodynamicRHS, :72-149 (2D).
inline void CalculateMorphodynamicRHS(const RunSet& rp, Grid& g, Tiles& tiles) {
    int nX = rp.nXpertile, nY = rp.nYpertile;
    double Hneps = rp.heightThreshold;
    for (int tID : g.activeTiles) {
        Tile& T = TL(tiles, tID);
        for (int i = 1; i <= nX; ++i)
            for (int j = 1; j <= nY; ++j) {
                double HnW = (i == 1) ? TL(tiles, T.West()).u(iHn, nX, j) : T.u(iHn, i - 1, j);
                double HnE = (i == nX) ? TL(tiles, T.East()).u(iHn, 1, j) : T.u(iHn, i + 1, j);
                double HnS = (j == 1) ? TL(tiles, T.South()).u(iHn, i, nY) : T.u(iHn, i, j - 1);
                double HnN = (j == nY) ? TL(tiles, T.North()).u(iHn, i, 1) : T.u(iHn, i, j + 1);
                if (T.u(iHn, i, j) < Hneps || HnW < Hneps || HnE < Hneps || HnS < Hneps || HnN < Hneps) {
                    for (int k = 1; k <= 4; ++k) T.ddtExplicit(k, i, j) = 0.0;
                    T.EminusD(i, j) = 0.0;
                } else {
                    double E, D;
                    ErosionDepositionTerms(rp, T.u.col(i, j), E, D);
                    T.EminusD(i, j) = E - D;
                }
            }
    }
    BtSourceTerm(rp, g, tiles);
}

// EqualiseTopographicBoundaryData, :588-687 (2D).
inline void EqualiseTopographicBoundaryData(const RunSet& rp, Grid& g, int tID) {
    int nX = rp.nXpertile, nY = rp.nYpertile;
    Tiles& tc = g.tileContainer;
    bool SW_updated = false, NE_updated = false;
    auto ok = [&](int id) { return InVector(g.activeTiles, id) || IsActiveGhostTile(g, id); };
    int ttW = g.tc(tID).West();
    if (ok(ttW)) {
        for (int j = 1; j <= nY; ++j) {
            g.tc(ttW).b0(nX + 1, j) = g.tc(tID).b0(1, j);
            g.tc(ttW).uPlusX(ib0, nX + 1, j) = g.tc(tID).uPlusX(ib0, 1, j);
            g.tc(ttW).uMinusX(ib0, nX + 1, j) = g.tc(tID).uMinusX(ib0, 1, j);
        }
        ComputeCellCentredTopographicData(rp, g, tc, ttW);
        int ttSW = g.tc(ttW).South();
        if (ok(ttSW)) {
            g.tc(ttSW).b0(nX + 1, nY + 1) = g.tc(tID).b0(1, 1);
            SW_updated = true;
            ComputeCellCentredTopographicData(rp, g, tc, ttSW);
        }
    }
    int ttE = g.tc(tID).East();
    if (ok(ttE)) {
        for (int j = 1; j <= nY; ++j) {
            g.tc(tID).b0(nX + 1, j) = g.tc(ttE).b0(1, j);
            g.tc(tID).uPlusX(ib0, nX + 1, j) = g.tc(ttE).uPlusX(ib0, 1, j);
            g.tc(tID).uMinusX(ib0, nX + 1, j) = g.tc(ttE).uMinusX(ib0, 1, j);
        }
        int ttNE = g.tc(ttE).North();
        if (ok(ttNE)) {
            g.tc(tID).b0(nX + 1, nY + 1) = g.tc(ttNE).b0(1, 1);
            NE_updated = true;
        }
        ComputeCellCentredTopographicData(rp, g, tc, tID);
    }
    int ttN = g.tc(tID).North();
    if (ok(ttN)) {
        for (int i = 1; i <= nX; ++i) {
            g.tc(tID).b0(i, nY + 1) = g.tc(ttN).b0(i, 1);
            g.tc(tID).uPlusY(ib0, i, nY + 1) = g.tc(ttN).uPlusY(ib0, i, 1);
            g.tc(tID).uMinusY(ib0, i, nY + 1) = g.tc(ttN).uMinusY(ib0, i, 1);
        }
        if (!NE_updated) {
            int ttNE = g.tc(ttN).East();
            if (ok(ttNE)) g.tc(tID).b0(nX + 1, nY + 1) = g.tc(ttNE).b0(1, 1);
        }
        ComputeCellCentredTopographicData(rp, g, tc, tID);
    }
    int ttS = g.tc(tID).South();
    if (ok(ttS)) {
        for (int i = 1; i <= nX; ++i) {
            g.tc(ttS).b0(i, nY + 1) = g.tc(tID).b0(i, 1);
            g.tc(ttS).uPlusY(ib0, i, nY + 1) = g.tc(tID).uPlusY(ib0, i, 1);
            g.tc(ttS).uMinusY(ib0, i, nY + 1) = g.tc(tID).uMinusY(ib0, i, 1);
        }
        ComputeCellCentredTopographicData(rp, g, tc, ttS);
        if (!SW_updated) {
            int ttSW = g.tc(ttS).West();
            if (ok(ttSW)) {
                g.tc(ttSW).b0(nX + 1, nY + 1) = g.tc(tID).b0(1, 1);
                ComputeCellCentredTopographicData(rp, g, tc, ttSW);
            }
        }
    }
}

// ---------------------------------------------------------------- UpdateTiles.f90
inline void SetPeriodicBoundaryConds(Grid& g, int k) {  // :521-566
    int gi, gj;
    GridCoords(k, g, gi, gj);
    Tile& T = g.tc(k);
    if (gi == 1) {
        T.neighbours[0] = TileID(g, g.nXtiles, gj);
        if (gj > 1 && gj < g.nYtiles) {
            T.cornertiles[0] = TileID(g, g.nXtiles, gj - 1);
            T.cornertiles[2] = TileID(g, g.nXtiles, gj + 1);
        } else if (gj == 1) {
            T.cornertiles[0] = TileID(g, g.nXtiles, g.nYtiles);
            T.cornertiles[2] = TileID(g, g.nXtiles, gj + 1);
        } else if (gj == g.nYtiles) {
            T.cornertiles[0] = TileID(g, g.nXtiles, gj - 1);
            T.cornertiles[2] = TileID(g, g.nXtiles, 1);
        }
    }
    if (gi == g.nXtiles) {
        T.neighbours[1] = TileID(g, 1, gj);
        if (gj > 1 && gj < g.nYtiles) {
            T.cornertiles[1] = TileID(g, 1, gj - 1);
            T.cornertiles[3] = TileID(g, 1, gj + 1);
        } else if (gj == 1) {
            T.cornertiles[1] = TileID(g, 1, g.nYtiles);
            T.cornertiles[3] = TileID(g, 1, gj + 1);
        } else if (gj == g.nYtiles) {
            T.cornertiles[1] = TileID(g, 1, gj - 1);
            T.cornertiles[3] = TileID(g, 1, 1);
        }
    }
    if (gj == 1) T.neighbours[3] = TileID(g, gi, g.nYtiles);
    if (gj == g.nYtiles) T.neighbours[2] = TileID(g, gi, 1);
}
inline void SetTileBoundaries(const RunSet& rp, Grid& g, int k) {  // :487-516
    Tile& T = g.tc(k);
    T.neighbours[0] = WestTile(k);
    T.neighbours[1] = EastTile(k);
    T.neighbours[2] = NorthTile(k, g);
    T.neighbours[3] = SouthTile(k, g);
    T.cornertiles[0] = WestTile(SouthTile(k, g));
    T.cornertiles[1] = EastTile(SouthTile(k, g));
    T.cornertiles[2] = WestTile(NorthTile(k, g));
    T.cornertiles[3] = EastTile(NorthTile(k, g));
    if (rp.bcs == KG_BC_PERIODIC) SetPeriodicBoundaryConds(g, k);
}
inline void AllocateU(const RunSet& rp, Grid& g, int k) {  // :221-268
    Tile& T = g.tc(k);
    int nX = rp.nXpertile, nY = rp.nYpertile;
    if (!T.u.allocated()) {
        T.u.allocate(ND, nX, nY, 0.0);
        for (int j = 1; j <= nY; ++j)
            for (int i = 1; i <= nX; ++i) T.u(irho, i, j) = rp.rhow;
    }
    if (!T.uLimX.allocated()) T.uLimX.allocate(ND, nX, nY, 0.0);
    if (!T.uLimY.allocated()) T.uLimY.allocate(ND, nX, nY, 0.0);
    if (!T.uPlusX.allocated()) T.uPlusX.allocate(ND, nX + 1, nY, 0.0);
    if (!T.uMinusX.allocated()) T.uMinusX.allocate(ND, nX + 1, nY, 0.0);
    if (!T.uPlusY.allocated()) T.uPlusY.allocate(ND, nX, nY + 1, 0.0);
    if (!T.uMinusY.allocated()) T.uMinusY.allocate(ND, nX, nY + 1, 0.0);
}
inline void AllocateTopographicData(const RunSet& rp, Grid& g, int k) {  // :271-337
    Tile& T = g.tc(k);
    int nX = rp.nXpertile, nY = rp.nYpertile;
    int gi, gj;
    GridCoords(k, g, gi, gj);
    double x, y;
    if (T.x.empty()) {
        T.x.resize(nX);
        for (int ii = 1; ii <= nX; ++ii) { GridToPhysical(rp, g, gi, gj, ii, 1, x, y); T.x[ii - 1] = x; }
        T.xmin = *std::min_element(T.x.begin(), T.x.end());
        T.xmax = *std::max_element(T.x.begin(), T.x.end());
    }
    if (T.y.empty()) {
        T.y.resize(nY);
        for (int jj = 1; jj <= nY; ++jj) { GridToPhysical(rp, g, gi, gj, 1, jj, x, y); T.y[jj - 1] = y; }
        T.ymin = *std::min_element(T.y.begin(), T.y.end());
        T.ymax = *std::max_element(T.y.begin(), T.y.end());
    }
    if (T.x_vertex.empty()) {
        T.x_vertex.resize(nX + 1);
        for (int ii = 1; ii <= nX; ++ii) T.x_vertex[ii - 1] = T.x[ii - 1] - 0.5 * rp.deltaX;
        T.x_vertex[nX] = T.x[nX - 1] + 0.5 * rp.deltaX;
    }
    if (T.y_vertex.empty()) {
        T.y_vertex.resize(nY + 1);
        for (int jj = 1; jj <= nY; ++jj) T.y_vertex[jj - 1] = T.y[jj - 1] - 0.5 * rp.deltaY;
        T.y_vertex[nY] = T.y[nY - 1] + 0.5 * rp.deltaY;
    }
    if (!T.b0.allocated()) T.b0.allocate(nX + 1, nY + 1, 0.0);
    if (!T.bt.allocated()) T.bt.allocate(nX + 1, nY + 1, 0.0);
    if (!T.EminusD.allocated()) T.EminusD.allocate(nX, nY, 0.0);
}
inline void SetDefaultTileData(const RunSet& rp, Grid& g, int k) {  // :647-664
    Tile& T = g.tc(k);
    for (int j = 1; j <= rp.nYpertile; ++j)
        for (int i = 1; i <= rp.nXpertile; ++i) {
            for (int d = 1; d <= 9; ++d) T.u(d, i, j) = 0.0;
            T.u(irho, i, j) = rp.rhow;
            T.u(iw, i, j) = T.u(ib0, i, j);
        }
}
inline void SetDomainBoundaryData(const RunSet& rp, Grid& g, int k) {  // :595-642
    Tile& T = g.tc(k);
    switch (rp.bcs) {
        case KG_BC_PERIODIC: return;
        case KG_BC_HALT:
        case KG_BC_SPONGE: SetDefaultTileData(rp, g, k); return;
        default: {
            double Hnval = rp.p.bcsHnval, uval = rp.p.bcsuval, vval = rp.p.bcsvval, psival = rp.p.bcspsival;
            double rho = Density(rp, psival);
            for (int i = 1; i <= rp.nXpertile; ++i)
                for (int j = 1; j <= rp.nYpertile; ++j) {
                    double hpval = Hnval / Gam(rp, T.u.col(i, j));
                    double w = T.u(ibt, i, j) + hpval;
                    w = w + T.u(ib0, i, j);
                    T.u(iw, i, j) = w;
                }
            for (int j = 1; j <= rp.nYpertile; ++j)
                for (int i = 1; i <= rp.nXpertile; ++i) {
                    T.u(irhoHnu, i, j) = rho * Hnval * uval;
                    T.u(irhoHnv, i, j) = rho * Hnval * vval;
                    T.u(iHnpsi, i, j) = Hnval * psival;
                    T.u(iHn, i, j) = Hnval;
                    T.u(iu, i, j) = uval;
                    T.u(iv, i, j) = vval;
                    T.u(ipsi, i, j) = psival;
                    T.u(irho, i, j) = rho;
                }
        }
    }
}
inline void UpdateGhostTileBCs(const RunSet& rp, Grid& g, int k) {  // :571-590
    if (OnDomainEdge(g, k)) SetDomainBoundaryData(rp, g, k);
    else SetDefaultTileData(rp, g, k);
}
// ReconstructwAtEdges, :669-750 (2D).
inline void ReconstructwAtEdges(const RunSet& rp, Grid& g, Tiles& tiles, int tID) {
    int nX = rp.nXpertile, nY = rp.nYpertile;
    double dx = g.deltaX, dy = g.deltaY;
    Tile& T = TL(tiles, tID);
    int nb = g.tc(tID).West();
    if (TileInBounds(g, nb) && TL(tiles, nb).TileOn) {
        for (int j = 1; j <= nY; ++j) CalculateLimitedDerivsBoundary(rp, g, iw, 1, j, tiles, tID, 'W');
        for (int j = 1; j <= nY; ++j) {
            T.uPlusX(iw, 1, j) = T.u(iw, 1, j) - T.uLimX(iw, 1, j) * 0.5 * dx;
            T.uMinusX(iw, 2, j) = T.u(iw, 1, j) + T.uLimX(iw, 1, j) * 0.5 * dx;
        }
    }
    nb = g.tc(tID).East();
    if (TileInBounds(g, nb) && TL(tiles, nb).TileOn) {
        for (int j = 1; j <= nY; ++j) CalculateLimitedDerivsBoundary(rp, g, iw, nX, j, tiles, tID, 'E');
        for (int j = 1; j <= nY; ++j) {
            T.uPlusX(iw, nX, j) = T.u(iw, nX, j) - T.uLimX(iw, nX, j) * 0.5 * dx;
            T.uMinusX(iw, nX + 1, j) = T.u(iw, nX, j) + T.uLimX(iw, nX, j) * 0.5 * dx;
        }
    }
    nb = g.tc(tID).South();
    if (TileInBounds(g, nb) && TL(tiles, nb).TileOn) {
        for (int i = 1; i <= nX; ++i) CalculateLimitedDerivsBoundary(rp, g, iw, i, 1, tiles, tID, 'S');
        for (int i = 1; i <= nX; ++i) {
            T.uPlusY(iw, i, 1) = T.u(iw, i, 1) - T.uLimY(iw, i, 1) * 0.5 * dy;
            T.uMinusY(iw, i, 2) = T.u(iw, i, 1) + T.uLimY(iw, i, 1) * 0.5 * dy;
        }
    }
    nb = g.tc(tID).North();
    if (TileInBounds(g, nb) && TL(tiles, nb).TileOn) {
        for (int i = 1; i <= nX; ++i) CalculateLimitedDerivsBoundary(rp, g, iw, i, nY, tiles, tID, 'N');
        for (int i = 1; i <= nX; ++i) {
            T.uPlusY(iw, i, nY) = T.u(iw, i, nY) - T.uLimY(iw, i, nY) * 0.5 * dy;
            T.uMinusY(iw, i, nY + 1) = T.u(iw, i, nY) + T.uLimY(iw, i, nY) * 0.5 * dy;
        }
    }
}
// AddGhostTiles, :389-481.
inline void AddGhostTiles(const RunSet& rp, Grid& g, int k) {
    std::vector<int> newGhost;
    int nIter = g.dim * 2 + 4 * (g.dim - 1);
    for (int i = 1; i <= nIter; ++i) {
        int tile;
        if (i > 4) {
            if (rp.bcs == KG_BC_PERIODIC) break;
            tile = g.tc(k).cornertiles[i - 5];
        } else {
            tile = g.tc(k).neighbours[i - 1];
        }
        if (!TileInBounds(g, tile)) throw KoError(KG_ERR_HALT_EDGE, "ghost tile outside the domain");
        bool already = (!g.ghostTiles.empty()) && InVector(g.ghostTiles, tile);
        if (already) {
            ReconstructwAtEdges(rp, g, g.tileContainer, tile);
        } else if (!g.tc(tile).TileOn && !InVector(newGhost, tile)) {
            newGhost.push_back(tile);
        }
    }
    if (newGhost.empty()) return;
    for (int t : newGhost) g.ghostTiles.push_back(t);
    for (int tile : newGhost) {
        AllocateU(rp, g, tile);
        AllocateTopographicData(rp, g, tile);
        SetTileBoundaries(rp, g, tile);
        GetHeights(rp, g, tile);
        ComputeCellCentredTopographicData(rp, g, g.tileContainer, tile);
        UpdateGhostTileBCs(rp, g, tile);
        ReconstructwAtEdges(rp, g, g.tileContainer, tile);
        g.tc(tile).isGhostTile = true;
    }
    for (int tile : newGhost) EqualiseTopographicBoundaryData(rp, g, tile);
}
inline void AllocateTile(const RunSet& rp, Grid& g, int k) {  // :120-219
    Tile& T = g.tc(k);
    T.TileOn = true;
    int nX = rp.nXpertile, nY = rp.nYpertile;
    if (!T.Hnmax.allocated()) T.Hnmax.allocate(nX, nY, 2, 0.0);
    if (!T.umax.allocated()) T.umax.allocate(nX, nY, 2, 0.0);
    if (!T.emax.allocated()) T.emax.allocate(nX, nY, 2, 0.0);
    if (!T.dmax.allocated()) T.dmax.allocate(nX, nY, 2, 0.0);
    if (!T.psimax.allocated()) T.psimax.allocate(nX, nY, 2, 0.0);
    if (!T.tfirst.allocated()) T.tfirst.allocate(nX, nY, -1.0);
    AllocateU(rp, g, k);
    SetTileBoundaries(rp, g, k);
    AllocateTopographicData(rp, g, k);
    GetHeights(rp, g, k);
    ComputeCellCentredTopographicData(rp, g, g.tileContainer, k);
    EqualiseTopographicBoundaryData(rp, g, k);
    Tile& U = g.tc(k);
    if (!U.hXFlux.allocated()) U.hXFlux.allocate(ND, nX + 1, nY, 0.0);
    if (!U.hYFlux.allocated()) U.hYFlux.allocate(ND, nX, nY + 1, 0.0);
    if (!U.gXFlux.allocated()) U.gXFlux.allocate(ND, nX + 1, nY, 0.0);
    if (!U.gYFlux.allocated()) U.gYFlux.allocate(ND, nX, nY + 1, 0.0);
    if (!U.pXFlux.allocated()) U.pXFlux.allocate(ND, nX + 1, nY, 0.0);
    if (!U.pYFlux.allocated()) U.pYFlux.allocate(ND, nX, nY + 1, 0.0);
    if (!U.ddtExplicit.allocated()) U.ddtExplicit.allocate(NFLUX, nX, nY, 0.0);
    if (!U.ddtImplicit.allocated()) U.ddtImplicit.allocate(NFLUX, nX, nY, 0.0);
    if (rp.MorphodynamicsOn && !U.ddtExplicitBt.allocated()) U.ddtExplicitBt.allocate(nX + 1, nY + 1, 0.0);
    U.containsSource = false;
}
inline void AddToActiveTiles(Grid& g, int k) {  // :81-117
    if (g.activeTiles.empty()) {
        g.activeTiles.push_back(k);
    } else if (!InVector(g.activeTiles, k)) {
        // AddToOrderedVector_i, src/utilities.f90:260-294
        size_t pos = 0;
        for (size_t i = 0; i < g.activeTiles.size(); ++i) {
            if (k < g.activeTiles[i]) break;
            pos++;
        }
        g.activeTiles.insert(g.activeTiles.begin() + (long)pos, k);
        if (g.ghostTiles.empty()) return;
        auto it = std::find(g.ghostTiles.begin(), g.ghostTiles.end(), k);
        if (it != g.ghostTiles.end()) {
            g.ghostTiles.erase(it);
            g.tc(k).isGhostTile = false;
        }
    }
}
inline void ActivateTile(const RunSet& rp, Grid& g, int k, bool restart = false) {  // :342-384
    Tile& T = g.tc(k);
    T.isGhostTile = false;
    if (!restart)  // a restart keeps the loaded w and bt (:361-370)
        for (int j = 1; j <= rp.nYpertile; ++j)
            for (int i = 1; i <= rp.nXpertile; ++i) {
                T.u(iw, i, j) = T.u(ib0, i, j);
                T.u(ibt, i, j) = 0.0;
            }
    AddGhostTiles(rp, g, k);
    Tiles& tc = g.tileContainer;
    ComputeInterfacialTopographicData(rp, g, tc, k);
    CalculateLimitedDerivs(rp, g, IFLUX, 4, tc, k);
    Reconstruct(rp, g, IFLUX, 4, true, tc, k);
    CorrectSlopes(rp, g, tc, k);
    ComputeDesingularisedVariables(rp, tc, k, true);
    CalculateLimitedDerivs(rp, g, IDESING, 5, tc, k);
    Reconstruct(rp, g, IDESING, 5, false, tc, k);
    double dummy = 100000.0;
    CalculateFluxes(rp, g, tc, k, dummy);
}
inline void AddTile(Grid& g, int tile, const RunSet& rp) {  // :56-78
    if (!TileInBounds(g, tile) || (OnDomainEdge(g, tile) && rp.bcs != KG_BC_PERIODIC)) {
        if (rp.bcs == KG_BC_HALT) throw KoError(KG_ERR_HALT_EDGE, "tried to add a tile outside the domain");
        return;
    }
    AddToActiveTiles(g, tile);
    AllocateTile(rp, g, tile);
    ActivateTile(rp, g, tile);
    g.xmin = std::min(g.tc(tile).xmin, g.xmin);
    g.xmax = std::max(g.tc(tile).xmax, g.xmax);
    g.ymin = std::min(g.tc(tile).ymin, g.ymin);
    g.ymax = std::max(g.tc(tile).ymax, g.ymax);
}

}  // namespace ko
