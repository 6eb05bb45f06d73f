// kg_morpho.cu -- the morphodynamic operator M (MorphodynamicTimeStepper,
// src/TimeStepper.f90:532-781) on sm_103a, FP64.
//
// M advances the vertex bed bt with the three-stage scheme and updates w and Hnpsi
// conservatively from the change in the cell-centred bed.  Per stage k = 1..3:
//   k_m_emd     E - D at every active cell of stage k-1, zero next to a dry cell
//               (CalculateMorphodynamicRHS, src/MorphodynamicRHS.f90:72-149)
//   k_m_bt      d(bt)/dt at every vertex of every active tile (BtSourceTerm, :154-305:
//               each tile updates its own copy of its edge vertices, with the reference's
//               Kahan orders, including the two pre-added entries at :210 and :266) and the
//               clamped stage update of bt
//   k_m_cells   cell-centred bed from the new vertices (ComputeCellCentredTopographicData),
//               the w / Hnpsi update (src/TimeStepper.f90:584-609) and the depth, solids
//               fraction and density of the stage (ComputeDesingularisedVariables without
//               velocities: u and v stay those the first hydraulic step left)
// then k_m_check evaluates the excess-deposition and 10 % depth-change tests (:709-753),
// k_m_redist_wave runs RedistributeGrid's ordered correction (src/Redistribute.f90) one
// dependency wave per launch, one warp per listed cell, and k_m_close ends the attempt
// (interfacial topography, M result, the FP32 form's factor cache).  Topography lives in
// two sets: the step-start bed (read-only here) and the bed M builds, so a refined attempt
// restarts from the step-start set.  The PLAIN / float instantiations are the FP32 form's.
#include <cuda_runtime.h>
#include "kg_engine.cuh"

namespace kg {

// cP is defined in kg_hydro.cu (one translation unit through kg_lib.cu).

constexpr int REDIST_THREADS = 512;

__device__ __forceinline__ size_t mp(int slot, int nf, int f, int npl) { return ((size_t)slot * nf + f) * (size_t)npl; }
// Plane f of the FP32 form's float stage planes (MF) of a slot.
__device__ __forceinline__ float* mfp(const DevArrays& A, int slot, int f, int SC) { return A.MF + mp(slot, MF_COUNT, f, SC); }

// FP32 form: 1/sqrt(x) from an FP32 seed and one Newton step (relative error about 1e-13,
// far below the form's FP32 error), and the step-start gamma of a cell from the
// topography-factor cache (gamma = gamma^2 / gamma).
__device__ __forceinline__ double rsqrt_nr(double x) {
    double y = (double)rsqrtf((float)x);
    return y * (1.5 - 0.5 * x * y * y);
}
// Bitwise equality of two doubles on the integer pipe (FP64 compares use the FP64 pipe,
// 1/64 of the FP32 rate on this GPU); differs from == only for +-0 and NaN.
__device__ __forceinline__ bool same_bits(double a, double b) { return __double_as_longlong(a) == __double_as_longlong(b); }
// x < e for e > 0 on the integer pipe: IEEE bit patterns of non-negative doubles order as
// their values and negative ones compare below every positive pattern (only a NaN with the
// sign bit set differs from the FP64 compare).
__device__ __forceinline__ bool below_pos(double x, double e) { return __double_as_longlong(x) < __double_as_longlong(e); }
__device__ __forceinline__ double gam_cached(const DevParams& P, const DevArrays& A, int ts, int s, int c, double bx, double by) {
    if (!P.geo) return 1.0;
    int SC = P.nX * P.nY;
    return (1.0 + (bx * bx + by * by)) * A.TD[ts][mp(s, 3, 2, SC) + c];
}
__device__ __forceinline__ double gam_nr(const DevParams& P, double bx, double by) {
    if (!P.geo) return 1.0;
    double g2 = 1.0 + (bx * bx + by * by);
    return g2 * rsqrt_nr(g2);
}

// Each step below is a per-item body (settings P / F, arrays A, slot s, item item_ of
// the tile, the tile's list position pos) called by a single-simulation kernel, which
// reads the constant bank, and by the batched kernels of kg_batch.cu, which read a
// per-member table.

// Copy the step-start bed into the M set and fill the stage state of im0 (the state the
// first hydraulic step produced).  ALT (FP32 form, fused stages): the stage depth and the
// six float stage planes go to their second copies, which the first fused stage reads.
template <bool PLAIN, bool ALT = false>
__device__ __forceinline__ void m_init(const DevParams& P, const DevParams32& F, const DevArrays& A, int s, int item_, int qa,
                                       int tcur, int tnew) {
    constexpr int hn_plane = ALT ? 3 : 2, alt = ALT ? MF_ALT : 0;
    int SC = P.nX * P.nY, SV = (P.nX + 1) * (P.nY + 1);
    // b0 (vertex plane 0, cell plane 0) is static and both topography sets hold it: only
    // the bed change and the slopes are carried into the M set.
    if (item_ < SV) {
        int v = item_;
        A.BV[tnew][mp(s, 2, 1, SV) + v] = A.BV[tcur][mp(s, 2, 1, SV) + v];
    }
    double e2 = P.hThr * P.hThr;
    if (item_ < SC) {
        int c = item_;
        double ct[4];
        ct[0] = A.CT[tcur][mp(s, 4, 0, SC) + c];
        for (int f = 1; f < 4; ++f) {
            ct[f] = A.CT[tcur][mp(s, 4, f, SC) + c];
            A.CT[tnew][mp(s, 4, f, SC) + c] = ct[f];
        }
        double w = A.Q[qa][mp(s, 4, 0, SC) + c], p = A.Q[qa][mp(s, 4, 3, SC) + c];
        double gam = PLAIN ? gam_cached(P, A, tcur, s, c, ct[2], ct[3]) : gam_of(P.geo, ct[2], ct[3]);
        double Hn = compute_hn(w, ct[0], ct[1], gam);
        if (PLAIN) {
            // the step-start quantities every stage and test of the attempt reuses
            double* Z = A.M0 + mp(s, 3, 0, SC) + c;
            Z[0] = Hn;
            Z[(size_t)SC] = Hn * gam;
            Z[2 * (size_t)SC] = p * gam;
        }
        double* M = A.MS + mp(s, 5, 0, SC) + c;
        M[0] = w;
        M[(size_t)SC] = p;
        // FP32 form: the stage depth is kept unclamped (the dry test reads its sign bit as a
        // value below the threshold, and the tests read it as the new depth)
        if (PLAIN) M[hn_plane * (size_t)SC] = Hn;
        if (Hn < 0.0) Hn = 0.0;
        double pp = p < 0.0 ? 0.0 : p;
        if (!PLAIN) M[2 * (size_t)SC] = Hn;
        if (PLAIN) {
            // the stage-0 inputs of the FP32 closures and of the vertex source, in float
            float Hf = (float)Hn, pf = (float)pp;
            float psi = fminf(2.f * Hf * pf / (Hf * Hf + fmaxf(Hf * Hf, (float)e2)), (float)P.maxPack);
            // (the float slopes of the step-start bed are the factor cache's)
            mfp(A, s, MF_PSI0, SC)[c] = psi;
            mfp(A, s, MF_HN + alt, SC)[c] = Hf;
            mfp(A, s, MF_PSI + alt, SC)[c] = psi;
            mfp(A, s, MF_RHO + alt, SC)[c] = density<float>(F, psi);
            mfp(A, s, MF_BT + alt, SC)[c] = (float)ct[1];
            mfp(A, s, MF_BX + alt, SC)[c] = A.TF[tcur][mp(s, 6, 1, SC) + c];
            mfp(A, s, MF_BY + alt, SC)[c] = A.TF[tcur][mp(s, 6, 2, SC) + c];
        } else {
            double psi = mn(2.0 * Hn * pp / (Hn * Hn + mx(Hn * Hn, e2)), P.maxPack);
            M[3 * (size_t)SC] = psi;
            M[4 * (size_t)SC] = density(P, psi);
        }
    }
}

// Depth of a cell of any tile as the M stage sees it: active tiles from the stage state,
// ghost tiles from their static data.
__device__ __forceinline__ double stage_hn(const DevArrays& A, int s, int c, int SC) {
    return A.kind[s] == SLOT_GHOST ? A.G9[mp(s, 9, 4, SC) + c] : A.MS[mp(s, 5, 2, SC) + c];
}

// FP32 form, shared by the per-item bodies and the fused stage (k_m_stage32), so both form
// every value with the same operations.  emd32: E - D of a wet cell (t, c) from its float
// stage planes (plane + off: the first or second copy) and slopes dbx, dby.
__device__ __forceinline__ float emd32(const DevParams& P, const DevParams32& F, const DevArrays& A, int t, int c, int SC,
                                       int off, float dbx, float dby) {
    Pt<float> pt{mfp(A, t, MF_HN + off, SC)[c], (float)A.UV[mp(t, 2, 0, SC) + c], (float)A.UV[mp(t, 2, 1, SC) + c],
                 mfp(A, t, MF_PSI + off, SC)[c], mfp(A, t, MF_RHO + off, SC)[c], mfp(A, t, MF_BT + off, SC)[c], dbx, dby,
                 gam_of<float>(P.geo, dbx, dby)};
    return erosion_minus_deposition<float>(F, pt);
}
// d(bt)/dt at a vertex from the E - D and slopes of its four cells (south-west, north-west,
// south-east, north-east), summed pairwise in FP32; the slopes only matter where E - D is
// non-zero around the vertex.
__device__ __forceinline__ float ddt32_vertex(const DevParams& P, const float ef[4], const float xf[4], const float yf[4]) {
    float kef = (ef[0] + ef[1]) + (ef[2] + ef[3]);
    if (kef == 0.f) return 0.f;
    float gx = 0.25f * ((xf[0] + xf[1]) + (xf[2] + xf[3])), gy = 0.25f * ((yf[0] + yf[1]) + (yf[2] + yf[3]));
    float gam = P.geo ? sqrtf(1.f + gx * gx + gy * gy) : 1.f;
    return -0.25f * gam * kef * (float)P.invSolid;
}
// The clamped stage update of a vertex's bt: the rate in FP32 (its E - D terms come from
// FP32 closures), the update as bt0 + a (bt_k - bt0 + dt ddt) in FP64, so a vertex with no
// erosion or deposition around it keeps its bed exactly.
__device__ __forceinline__ double bt32_stage(const DevParams& P, int stage, double bt0, double btp, double dt, float ddt32) {
    // No E - D around the vertex and no change in the earlier stages: every stage formula
    // gives bt0 + 0 (taken on the integer pipe: only -0 becomes +0).
    if (ddt32 == 0.f && (stage == 1 || same_bits(btp, bt0)))
        return mx(-P.EroDepth, same_bits(bt0, -0.0) ? 0.0 : bt0);
    double inc = (btp - bt0) + dt * (double)ddt32;
    double nb;
    if (stage == 1) nb = bt0 + dt * (double)ddt32;
    else if (stage == 2) nb = bt0 + 0.25 * inc;
    else nb = bt0 + (2.0 / 3.0) * inc;
    return mx(-P.EroDepth, nb);
}
// Cell c of slot s from its four new vertex bt values: the cell bed (static b0 parts from
// the cache, bt terms summed pairwise, differences first), the conservative w / Hnpsi
// update from the attempt's step-start cache with 1/gamma from an FP32-seeded Newton step,
// and the stage's depth (kept unclamped in MS plane hn_plane) and float closure inputs
// (planes + off).
__device__ __forceinline__ void cell32_update(const DevParams& P, const DevParams32& F, const DevArrays& A, int s, int c, int tcur,
                                              int tnew, double b00, double b10, double b01, double b11, int hn_plane, int off) {
    const int SC = P.nX * P.nY;
    const double psib = 1.0 - P.BedPorosity;
    // b0 is static: the cell b0 (the compensated sum of the set-up) and the b0 parts of the
    // slopes come from the cache; only the bt terms are summed here.
    double b0c = A.CT[tcur][mp(s, 4, 0, SC) + c];
    const double* B = A.B0S + mp(s, 2, 0, SC) + c;
    double btc = 0.25 * ((b00 + b10) + (b01 + b11));
    double dbx = B[0] + P.hdxR * ((b10 - b00) + (b11 - b01));
    double dby = B[(size_t)SC] + P.hdyR * ((b01 - b00) + (b11 - b10));
    A.CT[tnew][mp(s, 4, 1, SC) + c] = btc;
    A.CT[tnew][mp(s, 4, 2, SC) + c] = dbx;
    A.CT[tnew][mp(s, 4, 3, SC) + c] = dby;
    double gamnew = 1.0, ign = 1.0;
    if (P.geo) {
        double g2 = 1.0 + (dbx * dbx + dby * dby);
        ign = rsqrt_nr(g2);
        gamnew = g2 * ign;
    }
    double db = btc - A.CT[tcur][mp(s, 4, 1, SC) + c];
    // Hn gam and Hnpsi gam of the step start from the attempt's cache (m_init)
    const double* Z = A.M0 + mp(s, 3, 0, SC) + c;
    double w = (b0c + btc) + (Z[(size_t)SC] - db) * (ign * ign);
    double Hnpsi = (Z[2 * (size_t)SC] - psib * db) * ign;
    double Hn = ((w - b0c) - btc) * gamnew;
    double* M = A.MS + mp(s, 5, 0, SC) + c;
    M[0] = w;
    M[(size_t)SC] = Hnpsi;
    M[hn_plane * (size_t)SC] = Hn;  // unclamped (as m_init)
    if (Hn < 0.0) Hn = 0.0;
    float Hf = (float)Hn, pf = Hnpsi < 0.0 ? 0.f : (float)Hnpsi;
    float psif = fminf(2.f * Hf * pf / (Hf * Hf + fmaxf(Hf * Hf, F.hThr2)), F.maxPack);
    // the stage's inputs of the FP32 closures and of the vertex source, in float
    mfp(A, s, MF_HN + off, SC)[c] = Hf;
    mfp(A, s, MF_PSI + off, SC)[c] = psif;
    mfp(A, s, MF_RHO + off, SC)[c] = density<float>(F, psif);
    mfp(A, s, MF_BT + off, SC)[c] = (float)btc;
    mfp(A, s, MF_BX + off, SC)[c] = (float)dbx;
    mfp(A, s, MF_BY + off, SC)[c] = (float)dby;
}

// R = double: the FP64 drop-in; R = float: the FP32 form's closures (the depth test and
// the stored E - D stay FP64).
template <class R>
__device__ __forceinline__ void m_emd(const DevParams& P, const DevParams32& F, const DevArrays& A, int s, int item_, int tnew) {
    int nX = P.nX, nY = P.nY, SC = nX * nY;
    int sW = A.nbr[s * 8 + NB_W], sE = A.nbr[s * 8 + NB_E], sN = A.nbr[s * 8 + NB_N], sS = A.nbr[s * 8 + NB_S];
    const double* CT = A.CT[tnew];
    if (item_ < SC) {
        int c = item_;
        int i = c % nX, j = c / nX;
        double Hn = A.MS[mp(s, 5, 2, SC) + c];
        double HnW = (i == 0) ? stage_hn(A, sW, j * nX + nX - 1, SC) : A.MS[mp(s, 5, 2, SC) + c - 1];
        double HnE = (i == nX - 1) ? stage_hn(A, sE, j * nX, SC) : A.MS[mp(s, 5, 2, SC) + c + 1];
        double HnS = (j == 0) ? stage_hn(A, sS, (nY - 1) * nX + i, SC) : A.MS[mp(s, 5, 2, SC) + c - nX];
        double HnN = (j == nY - 1) ? stage_hn(A, sN, i, SC) : A.MS[mp(s, 5, 2, SC) + c + nX];
        double e = P.hThr;
        double emd = 0.0;
        bool dry;
        if constexpr (sizeof(R) == sizeof(float))
            dry = below_pos(Hn, e) || below_pos(HnW, e) || below_pos(HnE, e) || below_pos(HnS, e) || below_pos(HnN, e);
        else
            dry = Hn < e || HnW < e || HnE < e || HnS < e || HnN < e;
        if constexpr (sizeof(R) == sizeof(float)) {
            // the FP32 form: the stage's closure inputs from the float planes, E - D kept in float
            float e = 0.f;
            if (!dry) e = emd32(P, F, A, s, c, SC, 0, mfp(A, s, MF_BX, SC)[c], mfp(A, s, MF_BY, SC)[c]);
            mfp(A, s, MF_EMD, SC)[c] = e;
        } else {
            if (!dry) {
                R dbx = (R)CT[mp(s, 4, 2, SC) + c], dby = (R)CT[mp(s, 4, 3, SC) + c];
                Pt<R> pt{(R)Hn, (R)A.UV[mp(s, 2, 0, SC) + c], (R)A.UV[mp(s, 2, 1, SC) + c], (R)A.MS[mp(s, 5, 3, SC) + c],
                         (R)A.MS[mp(s, 5, 4, SC) + c], (R)CT[mp(s, 4, 1, SC) + c], dbx, dby, gam_of<R>(P.geo, dbx, dby)};
                emd = erosion_minus_deposition<R>(P, pt);
            }
            A.EMD[(size_t)s * SC + c] = emd;
        }
    }
}

// Cell value of one of the eight tiles around (and including) a tile: field f of CT
// (2: dbdx, 3: dbdy) or EMD (f = -1) at tile-local (i, j).
__device__ __forceinline__ double cellv(const DevArrays& A, const double* CT, int s, int f, int i, int j, int nX, int SC) {
    if (s < 0) return 0.0;  // a diagonal tile that was never allocated (periodic corners)
    size_t c = (size_t)j * nX + i;
    return f < 0 ? A.EMD[(size_t)s * SC + c] : CT[mp(s, 4, f, SC) + c];
}

// Vertex source term and clamped stage update of bt.  PLAIN (the FP32 form) sums the four
// cell terms pairwise instead of the reference's compensated sums.
template <bool PLAIN>
__device__ __forceinline__ void m_bt(const DevParams& P, const DevArrays& A, int s, int item_, int tcur, int tnew, int stage,
                                     double dt) {
    int nX = P.nX, nY = P.nY, SC = nX * nY, SV = (nX + 1) * (nY + 1);
    const double* CT = A.CT[tnew];
    int sW = A.nbr[s * 8 + NB_W], sE = A.nbr[s * 8 + NB_E], sN = A.nbr[s * 8 + NB_N], sS = A.nbr[s * 8 + NB_S];
    int sSW = sW < 0 ? -1 : A.nbr[sW * 8 + NB_S], sSE = sE < 0 ? -1 : A.nbr[sE * 8 + NB_S];
    int sNW = sW < 0 ? -1 : A.nbr[sW * 8 + NB_N], sNE = sE < 0 ? -1 : A.nbr[sE * 8 + NB_N];
    double psib = 1.0 - P.BedPorosity;
    if (item_ < SV) {
        int v = item_;
        int a = v % (nX + 1), b = v / (nX + 1);  // vertex (a, b), 0-based
        // The four cells around the vertex in the reference's list order, as (slot, i, j).
        int cs[4], ci[4], cj[4];
        int mode = 0;  // 0 plain, 1 west edge (E-D list pre-adds its last two), 2 NE corner (dbdx pre-add)
        if (a > 0 && a < nX && b > 0 && b < nY) {
            cs[0] = s; ci[0] = a - 1; cj[0] = b - 1;
            cs[1] = s; ci[1] = a - 1; cj[1] = b;
            cs[2] = s; ci[2] = a;     cj[2] = b - 1;
            cs[3] = s; ci[3] = a;     cj[3] = b;
        } else if (a == 0 && b > 0 && b < nY) {
            cs[0] = sW; ci[0] = nX - 1; cj[0] = b - 1;
            cs[1] = sW; ci[1] = nX - 1; cj[1] = b;
            cs[2] = s;  ci[2] = 0;      cj[2] = b - 1;
            cs[3] = s;  ci[3] = 0;      cj[3] = b;
            mode = 1;
        } else if (a == nX && b > 0 && b < nY) {
            cs[0] = s;  ci[0] = nX - 1; cj[0] = b - 1;
            cs[1] = s;  ci[1] = nX - 1; cj[1] = b;
            cs[2] = sE; ci[2] = 0;      cj[2] = b - 1;
            cs[3] = sE; ci[3] = 0;      cj[3] = b;
        } else if (b == nY && a > 0 && a < nX) {
            cs[0] = s;  ci[0] = a - 1; cj[0] = nY - 1;
            cs[1] = sN; ci[1] = a - 1; cj[1] = 0;
            cs[2] = s;  ci[2] = a;     cj[2] = nY - 1;
            cs[3] = sN; ci[3] = a;     cj[3] = 0;
        } else if (b == 0 && a > 0 && a < nX) {
            cs[0] = sS; ci[0] = a - 1; cj[0] = nY - 1;
            cs[1] = s;  ci[1] = a - 1; cj[1] = 0;
            cs[2] = sS; ci[2] = a;     cj[2] = nY - 1;
            cs[3] = s;  ci[3] = a;     cj[3] = 0;
        } else if (a == 0 && b == 0) {
            cs[0] = sSW; ci[0] = nX - 1; cj[0] = nY - 1;
            cs[1] = sW;  ci[1] = nX - 1; cj[1] = 0;
            cs[2] = sS;  ci[2] = 0;      cj[2] = nY - 1;
            cs[3] = s;   ci[3] = 0;      cj[3] = 0;
        } else if (a == nX && b == 0) {
            cs[0] = sS;  ci[0] = nX - 1; cj[0] = nY - 1;
            cs[1] = s;   ci[1] = nX - 1; cj[1] = 0;
            cs[2] = sSE; ci[2] = 0;      cj[2] = nY - 1;
            cs[3] = sE;  ci[3] = 0;      cj[3] = 0;
        } else if (a == 0 && b == nY) {
            cs[0] = sW;  ci[0] = nX - 1; cj[0] = nY - 1;
            cs[1] = sNW; ci[1] = nX - 1; cj[1] = 0;
            cs[2] = s;   ci[2] = 0;      cj[2] = nY - 1;
            cs[3] = sN;  ci[3] = 0;      cj[3] = 0;
        } else {  // NE
            cs[0] = s;   ci[0] = nX - 1; cj[0] = nY - 1;
            cs[1] = sN;  ci[1] = nX - 1; cj[1] = 0;
            cs[2] = sE;  ci[2] = 0;      cj[2] = nY - 1;
            cs[3] = sNE; ci[3] = 0;      cj[3] = 0;
            mode = 2;
        }
        double x[4], y[4], e[4];
        double kx = 0.0, ky = 0.0, ke = 0.0;
        float ddt32 = 0.f;
        if (PLAIN) {
            // FP32 form: the four cells' E - D and slopes from the float stage planes (a ghost
            // cell's E - D is zero and its slopes are the step-start factor cache's).
            float ef[4], xf[4] = {0.f, 0.f, 0.f, 0.f}, yf[4] = {0.f, 0.f, 0.f, 0.f};
            for (int q = 0; q < 4; ++q) ef[q] = cs[q] < 0 ? 0.f : mfp(A, cs[q], MF_EMD, SC)[cj[q] * nX + ci[q]];
            if ((ef[0] + ef[1]) + (ef[2] + ef[3]) != 0.f) {
                for (int q = 0; q < 4; ++q) {
                    int cc = cj[q] * nX + ci[q];
                    if (cs[q] < 0) {
                        xf[q] = 0.f;
                        yf[q] = 0.f;
                    } else if (A.kind[cs[q]] == SLOT_ACTIVE) {
                        xf[q] = mfp(A, cs[q], MF_BX, SC)[cc];
                        yf[q] = mfp(A, cs[q], MF_BY, SC)[cc];
                    } else {
                        xf[q] = A.TF[tcur][mp(cs[q], 6, 1, SC) + cc];
                        yf[q] = A.TF[tcur][mp(cs[q], 6, 2, SC) + cc];
                    }
                }
            }
            ddt32 = ddt32_vertex(P, ef, xf, yf);
        } else {
            for (int q = 0; q < 4; ++q) e[q] = cellv(A, CT, cs[q], -1, ci[q], cj[q], nX, SC);
            for (int q = 0; q < 4; ++q) {
                x[q] = cellv(A, CT, cs[q], 2, ci[q], cj[q], nX, SC);
                y[q] = cellv(A, CT, cs[q], 3, ci[q], cj[q], nX, SC);
            }
            kx = (mode == 2) ? kahan3(x[0], x[1], x[2] + x[3]) : kahan4(x[0], x[1], x[2], x[3]);
            ky = kahan4(y[0], y[1], y[2], y[3]);
            ke = (mode == 1) ? kahan3(e[0], e[1], e[2] + e[3]) : kahan4(e[0], e[1], e[2], e[3]);
        }
        double bt0 = A.BV[tcur][mp(s, 2, 1, SV) + v];
        double btp = A.BV[tnew][mp(s, 2, 1, SV) + v];
        double nb;
        if (PLAIN) {
            A.BV[tnew][mp(s, 2, 1, SV) + v] = bt32_stage(P, stage, bt0, btp, dt, ddt32);
            return;
        } else {
            double gam = gam_of(P.geo, 0.25 * kx, 0.25 * ky);
            double ddt = -0.25 * gam / psib * ke;
            if (stage == 1) nb = bt0 + dt * ddt;
            else if (stage == 2) nb = 0.75 * bt0 + 0.25 * (btp + dt * ddt);
            else nb = (1.0 / 3.0) * bt0 + (2.0 / 3.0) * (btp + dt * ddt);
        }
        A.BV[tnew][mp(s, 2, 1, SV) + v] = mx(-P.EroDepth, nb);
    }
}

// Cell-centred bed of stage k, the conservative w / Hnpsi update and the stage's depth,
// solids fraction and density.  PLAIN (the FP32 form) takes the vertex sums pairwise
// (differences first) and one divide per cell; every quantity stays FP64.
template <bool PLAIN>
__device__ __forceinline__ void m_cells(const DevParams& P, const DevParams32& F, const DevArrays& A, int s, int item_, int qa,
                                        int tcur, int tnew) {
    int nX = P.nX, nY = P.nY, SC = nX * nY, SV = (nX + 1) * (nY + 1);
    const double* b0 = A.BV[tnew] + mp(s, 2, 0, SV);
    const double* bt = A.BV[tnew] + mp(s, 2, 1, SV);
    double psib = 1.0 - P.BedPorosity, e2 = P.hThr * P.hThr;
    if (item_ < SC) {
        int c = item_;
        int i = c % nX, j = c / nX;
        int v00 = j * (nX + 1) + i, v10 = v00 + 1, v01 = v00 + (nX + 1), v11 = v01 + 1;
        if (PLAIN) {
            // FP32 form: a cell whose four vertices kept their bed, and whose cell bed in
            // the M set is still the step-start one, keeps its current stage state.
            const double* bt0 = A.BV[tcur] + mp(s, 2, 1, SV);
            const double *C0 = A.CT[tcur], *C3 = A.CT[tnew];
            if (same_bits(bt[v00], bt0[v00]) && same_bits(bt[v10], bt0[v10]) && same_bits(bt[v01], bt0[v01]) &&
                same_bits(bt[v11], bt0[v11]) && same_bits(C3[mp(s, 4, 1, SC) + c], C0[mp(s, 4, 1, SC) + c]) &&
                same_bits(C3[mp(s, 4, 2, SC) + c], C0[mp(s, 4, 2, SC) + c]) && same_bits(C3[mp(s, 4, 3, SC) + c], C0[mp(s, 4, 3, SC) + c]))
                return;
        }
        if (PLAIN) {
            cell32_update(P, F, A, s, c, tcur, tnew, bt[v00], bt[v10], bt[v01], bt[v11], 2, 0);
            return;
        }
        double b0c = 0.25 * kahan4(b0[v00], b0[v10], b0[v01], b0[v11]);
        double btc = 0.25 * kahan4(bt[v00], bt[v10], bt[v01], bt[v11]);
        double ax[8] = {b0[v10], bt[v10], -b0[v00], -bt[v00], b0[v11], bt[v11], -b0[v01], -bt[v01]};
        double ay[8] = {b0[v01], bt[v01], -b0[v00], -bt[v00], b0[v11], bt[v11], -b0[v10], -bt[v10]};
        double dbx = 0.5 * P.dxR * kahan8(ax);
        double dby = 0.5 * P.dyR * kahan8(ay);
        A.CT[tnew][mp(s, 4, 0, SC) + c] = b0c;
        A.CT[tnew][mp(s, 4, 1, SC) + c] = btc;
        A.CT[tnew][mp(s, 4, 2, SC) + c] = dbx;
        A.CT[tnew][mp(s, 4, 3, SC) + c] = dby;
        const double* C0 = A.CT[tcur];
        double gamold = gam_of(P.geo, C0[mp(s, 4, 2, SC) + c], C0[mp(s, 4, 3, SC) + c]);
        double gamnew = gam_of(P.geo, dbx, dby);
        double db = btc - C0[mp(s, 4, 1, SC) + c];
        double w0 = A.Q[qa][mp(s, 4, 0, SC) + c], p0 = A.Q[qa][mp(s, 4, 3, SC) + c];
        double Hn_old = compute_hn(w0, C0[mp(s, 4, 0, SC) + c], C0[mp(s, 4, 1, SC) + c], gamold);
        double w = -db / gamnew / gamnew;
        w = w + btc;
        w = w + Hn_old * gamold / gamnew / gamnew;
        w = w + b0c;
        double Hnpsi = -(psib)*db / gamnew;
        Hnpsi = Hnpsi + p0 * gamold / gamnew;
        double Hn = compute_hn(w, b0c, btc, gamnew);
        if (Hn < 0.0) Hn = 0.0;
        double pp = Hnpsi < 0.0 ? 0.0 : Hnpsi;
        double psi = mn(2.0 * Hn * pp / (Hn * Hn + mx(Hn * Hn, e2)), P.maxPack);
        double* M = A.MS + mp(s, 5, 0, SC) + c;
        M[0] = w;
        M[(size_t)SC] = Hnpsi;
        M[2 * (size_t)SC] = Hn;
        M[3 * (size_t)SC] = psi;
        M[4 * (size_t)SC] = density(P, psi);
    }
}

// ExcessDeposition (src/Redistribute.f90:158-198) of cell (s, c) between im0 and im3.
// PLAIN (the FP32 form) takes gamma from the factor cache / an FP32-seeded Newton step.
// STAGE_HN (FP32 form, the check after the stages): the new depth is the stage's unclamped
// depth, which m_cells formed with the same operations from the same w, bed and gamma (and
// which m_init set for a cell no stage changed, one the check skips); the redistribution
// walk, which changes cells after the stages, recomputes it.
template <bool PLAIN = false, bool STAGE_HN = false>
__device__ __forceinline__ void excess_deposition(const DevParams& P, const DevArrays& A, int s, int c, int qa, int tcur,
                                                  int tnew, double& excess, double& deltaBt, double& psiold,
                                                  double& Hn_old, double& Hn_new) {
    int SC = P.nX * P.nY;
    const double *C0 = A.CT[tcur], *C3 = A.CT[tnew];
    if (PLAIN) {
        // the step-start Hn, Hn gam, Hnpsi gam and psi from the attempt's cache (m_init)
        const double* Z = A.M0 + mp(s, 3, 0, SC) + c;
        Hn_old = Z[0];
        if (STAGE_HN) {
            Hn_new = A.MS[mp(s, 5, 2, SC) + c];
        } else {
            double gamnew = gam_nr(P, C3[mp(s, 4, 2, SC) + c], C3[mp(s, 4, 3, SC) + c]);
            Hn_new = compute_hn(A.MS[mp(s, 5, 0, SC) + c], C3[mp(s, 4, 0, SC) + c], C3[mp(s, 4, 1, SC) + c], gamnew);
        }
        deltaBt = C3[mp(s, 4, 1, SC) + c] - C0[mp(s, 4, 1, SC) + c];
        psiold = (double)A.MF[(size_t)s * SC + c];
        // The deposition of this attempt is limited by the solids and depth the cell holds,
        // taken at 0 where they are negative: next to deep flows the FP32 fluxes leave
        // round-off of order 1e-9 in thin cells, which can make Hnpsi or the depth slightly
        // negative, and a deficit the attempt did not cause is not excess deposition (M could
        // never remove it, and refining dt would not shrink it).  Where both are >= 0 this is
        // the reference's formula.
        excess = -(mx(Z[2 * (size_t)SC], 0.0) * P.invSolid - deltaBt);
        excess = mx(excess, -(mx(Z[(size_t)SC], 0.0) - deltaBt));
        return;
    }
    double gamold = gam_of(P.geo, C0[mp(s, 4, 2, SC) + c], C0[mp(s, 4, 3, SC) + c]);
    double gamnew = gam_of(P.geo, C3[mp(s, 4, 2, SC) + c], C3[mp(s, 4, 3, SC) + c]);
    double w0 = A.Q[qa][mp(s, 4, 0, SC) + c], p0 = A.Q[qa][mp(s, 4, 3, SC) + c];
    Hn_old = compute_hn(w0, C0[mp(s, 4, 0, SC) + c], C0[mp(s, 4, 1, SC) + c], gamold);
    Hn_new = compute_hn(A.MS[mp(s, 5, 0, SC) + c], C3[mp(s, 4, 0, SC) + c], C3[mp(s, 4, 1, SC) + c], gamnew);
    deltaBt = C3[mp(s, 4, 1, SC) + c] - C0[mp(s, 4, 1, SC) + c];
    // im0's solids fraction as the first hydraulic step left it
    double H0 = Hn_old < 0.0 ? 0.0 : Hn_old, pp = p0 < 0.0 ? 0.0 : p0, e2 = P.hThr * P.hThr;
    psiold = mn(2.0 * H0 * pp / (H0 * H0 + mx(H0 * H0, e2)), P.maxPack);
    excess = -(p0 * gamold / (1.0 - P.BedPorosity) - deltaBt);
    excess = mx(excess, -(Hn_old * gamold - deltaBt));
}

// The two tests of src/TimeStepper.f90:709-753 for every active cell.  flags[0] is set
// when the step must be refined; redistribution candidates are appended with their loop
// position (tile position in the active list, then j, then i) so the host can order them.
template <bool PLAIN>
__device__ __forceinline__ void m_check(const DevParams& P, const DevArrays& A, int s, int item_, int pos, int qa, int tcur,
                                        int tnew, int* flags, unsigned long long* cand_key, double* cand_ex, int* ncand,
                                        int cand_cap) {
    int SC = P.nX * P.nY;
    if (item_ < SC) {
        int c = item_;
        if (PLAIN) {
            // A cell whose bed, slopes and free surface M left as they were has no excess
            // (its bed change is 0) and no depth change: neither test can fire.
            const double *C0 = A.CT[tcur], *C3 = A.CT[tnew];
            if (same_bits(C3[mp(s, 4, 1, SC) + c], C0[mp(s, 4, 1, SC) + c]) &&
                same_bits(C3[mp(s, 4, 2, SC) + c], C0[mp(s, 4, 2, SC) + c]) &&
                same_bits(C3[mp(s, 4, 3, SC) + c], C0[mp(s, 4, 3, SC) + c]) &&
                same_bits(A.MS[mp(s, 5, 0, SC) + c], A.Q[qa][mp(s, 4, 0, SC) + c]))
                return;
        }
        double ex, dBt, psiold, Hn_old, Hn_new;
        excess_deposition<PLAIN, PLAIN>(P, A, s, c, qa, tcur, tnew, ex, dBt, psiold, Hn_old, Hn_new);
        bool refine = false;
        if (ex > kEPS && dBt > kEPS && psiold > -kEPS) {
            if (Hn_old < P.EroCriticalHeight || fabs(Hn_new - Hn_old) < P.EroCriticalHeight) {
                int k = atomicAdd(ncand, 1);
                if (k < cand_cap) {
                    cand_key[k] = ((unsigned long long)pos << 32) | (unsigned long long)c;
                    cand_ex[k] = ex;
                }
            } else {
                refine = true;
            }
        } else if (!(Hn_old < P.EroCriticalHeight)) {
            if (PLAIN) {
                if (fabs(Hn_new - Hn_old) > 0.1 * fabs(Hn_old)) refine = true;
            } else {
                double rel = fabs(Hn_new - Hn_old) / fabs(Hn_old);
                if (rel > 0.1) refine = true;
            }
        }
        if (refine) atomicOr(flags, 1);
    }
}

// Kahan-ordered cell-centred bed of one cell from the M set (ComputeCellCentredTopographic-
// Data_ij, src/MorphodynamicRHS.f90:371-414: bt, dbdx, dbdy; b0 is left as it is).
__device__ void cell_topo_ij(const DevParams& P, const DevArrays& A, int tnew, int s, int i, int j, double* out3 = nullptr) {
    int nX = P.nX, SC = nX * P.nY, SV = (nX + 1) * (P.nY + 1);
    const double* b0 = A.BV[tnew] + mp(s, 2, 0, SV);
    const double* bt = A.BV[tnew] + mp(s, 2, 1, SV);
    int v00 = j * (nX + 1) + i, v10 = v00 + 1, v01 = v00 + (nX + 1), v11 = v01 + 1;
    size_t c = (size_t)j * nX + i;
    double btc = 0.25 * kahan4(bt[v00], bt[v10], bt[v01], bt[v11]);
    double ax[8] = {b0[v10], bt[v10], -b0[v00], -bt[v00], b0[v11], bt[v11], -b0[v01], -bt[v01]};
    double ay[8] = {b0[v01], bt[v01], -b0[v00], -bt[v00], b0[v11], bt[v11], -b0[v10], -bt[v10]};
    double dbx = 0.5 * P.dxR * kahan8(ax), dby = 0.5 * P.dyR * kahan8(ay);
    A.CT[tnew][mp(s, 4, 1, SC) + c] = btc;
    A.CT[tnew][mp(s, 4, 2, SC) + c] = dbx;
    A.CT[tnew][mp(s, 4, 3, SC) + c] = dby;
    if (out3) { out3[0] = btc; out3[1] = dbx; out3[2] = dby; }
}

__device__ __forceinline__ void set_bt(const DevArrays& A, int tnew, int s, int a, int b, double v, int SV, int nX) {
    // Only active tiles' copies persist; a ghost tile keeps its static bed.
    if (s >= 0 && A.kind[s] == SLOT_ACTIVE) A.BV[tnew][mp(s, 2, 1, SV) + (size_t)b * (nX + 1) + a] = v;
}

// RedistributeCell, src/Redistribute.f90:249-475, up to the corrected vertices (:249-399);
// the cells are updated by redist_cell.  Returns false when the cell borders no
// depositional vertex.
// PLAIN (the FP32 form) takes gamma from the factor cache, sums without compensation and
// multiplies by 1 / (1 - porosity): a shorter FP64 chain for the serial walk.
template <bool PLAIN>
__device__ bool redistribute_cell(const DevParams& P, const DevArrays& A, int qa, int tcur, int tnew, int s, int i, int j,
                                  double corr) {
    int nX = P.nX, nY = P.nY, SC = nX * nY, SV = (nX + 1) * (nY + 1);
    const double* bt0 = A.BV[tcur] + mp(s, 2, 1, SV);
    double* bt3 = A.BV[tnew] + mp(s, 2, 1, SV);
    int N = 0;
    double sum = 0.0, bd[4] = {0, 0, 0, 0};
    int di[4], dj[4];
    const int ca[4] = {i, i + 1, i, i + 1}, cb[4] = {j, j, j + 1, j + 1};
    for (int q = 0; q < 4; ++q) {
        int v = cb[q] * (nX + 1) + ca[q];
        bd[N] = bt3[v] - bt0[v];
        if (bd[N] > 0.0) {
            di[N] = ca[q];
            dj[N] = cb[q];
            sum = sum + bd[N];
            N = N + 1;
        }
    }
    if (N == 0) return false;
    double delta = 4.0 * corr / sum;
    const double *C0 = A.CT[tcur], *C3 = A.CT[tnew];
    size_t c = (size_t)j * nX + i;
    // Hg: the step-start Hn (clamped at 0) times gam; Hgp: Hnpsi gam / (1 - porosity).  The
    // FP32 form takes both from the attempt's cache (m_init).
    double Hg, Hgp;
    if (PLAIN) {
        const double* Z = A.M0 + mp(s, 3, 0, SC) + c;
        Hg = Z[0] < 0.0 ? 0.0 : Z[(size_t)SC];
        Hgp = mx(Z[2 * (size_t)SC], 0.0) * P.invSolid;  // as the excess test: negative solids taken at 0
    } else {
        double gamold = gam_of(P.geo, C0[mp(s, 4, 2, SC) + c], C0[mp(s, 4, 3, SC) + c]);
        double w0 = A.Q[qa][mp(s, 4, 0, SC) + c];
        double Hnold = compute_hn(w0, C0[mp(s, 4, 0, SC) + c], C0[mp(s, 4, 1, SC) + c], gamold);
        if (Hnold < 0.0) Hnold = 0.0;
        Hg = Hnold * gamold;
        Hgp = A.Q[qa][mp(s, 4, 3, SC) + c] * gamold / (1.0 - P.BedPorosity);
    }
    double db = C3[mp(s, 4, 1, SC) + c] - C0[mp(s, 4, 1, SC) + c];
    double tol = kEPS * A.MS[mp(s, 5, 0, SC) + c] * 10.0;
    double adjustment = 0.0;
    double disc = PLAIN ? (Hg - db) + corr : kahan3(Hg, -db, corr);
    if (fabs(disc) < tol) {
        adjustment = PLAIN ? (tol - Hg) + db : kahan3(tol, -Hg, db);
        adjustment = adjustment * (4.0 / sum);
        adjustment = adjustment - delta;
        adjustment = mx(adjustment, 0.0);
    }
    tol = kEPS * 10.0;
    disc = PLAIN ? (Hgp - db) + corr : kahan3(Hgp, -db, corr);
    if (fabs(disc) < tol) {
        double ap = PLAIN ? (tol - Hgp) + db : kahan3(tol, -Hgp, db);
        ap = ap * (4.0 / sum);
        ap = ap - delta;
        adjustment = mx(adjustment, ap);
    }
    delta = delta + adjustment;
    int sW = A.nbr[s * 8 + NB_W], sE = A.nbr[s * 8 + NB_E], sN = A.nbr[s * 8 + NB_N], sS = A.nbr[s * 8 + NB_S];
    for (int k = 0; k < N; ++k) {
        int v = dj[k] * (nX + 1) + di[k];
        bt3[v] = bt3[v] - delta * bd[k];
        double val = bt3[v];
        if (di[k] == 0) set_bt(A, tnew, sW, nX, dj[k], val, SV, nX);
        else if (di[k] == nX) set_bt(A, tnew, sE, 0, dj[k], val, SV, nX);
        if (dj[k] == 0) {
            set_bt(A, tnew, sS, di[k], nY, val, SV, nX);
            if (di[k] == 0 && sS >= 0) set_bt(A, tnew, A.nbr[sS * 8 + NB_W], nX, nY, val, SV, nX);
            if (di[k] == nX && sS >= 0) set_bt(A, tnew, A.nbr[sS * 8 + NB_E], 0, nY, val, SV, nX);
        }
        if (dj[k] == nY) {
            set_bt(A, tnew, sN, di[k], 0, val, SV, nX);
            if (di[k] == 0 && sN >= 0) set_bt(A, tnew, A.nbr[sN * 8 + NB_W], nX, 0, val, SV, nX);
            if (di[k] == nX && sN >= 0) set_bt(A, tnew, A.nbr[sN * 8 + NB_E], 0, 0, val, SV, nX);
        }
    }
    return true;
}

// The 3 x 3 cells a redistribution at cell (s, i, j) updates, column by column from the
// west as the reference's navigation visits them (:404-448; i, j 0-based).  Each column's
// tile is s or its west/east neighbour, and a cell above or below it lies in that tile's
// north/south neighbour, which is what the reference's walk reaches when every tile
// exists.  vt[k] = -1 for a cell whose tile was never allocated: on periodic domains the
// diagonal tiles get no ghost copy (src/UpdateTiles.f90:415-418), and only that tile's
// cells are skipped.
__device__ __forceinline__ void redist_cells_of(const DevParams& P, const DevArrays& A, int s, int i, int j, int vt[9], int vi[9],
                                                int vj[9]) {
    int nX = P.nX, nY = P.nY;
    int sW = A.nbr[s * 8 + NB_W], sE = A.nbr[s * 8 + NB_E];
    int n = 0;
    for (int di = -1; di <= 1; ++di) {
        int ci = i + di, col = s;
        if (ci < 0) { col = sW; ci += nX; }
        else if (ci >= nX) { col = sE; ci -= nX; }
        for (int dj = -1; dj <= 1; ++dj) {
            int cj = j + dj, ct = col;
            if (cj < 0) { ct = col < 0 ? -1 : A.nbr[col * 8 + NB_S]; cj += nY; }
            else if (cj >= nY) { ct = col < 0 ? -1 : A.nbr[col * 8 + NB_N]; cj -= nY; }
            vt[n] = ct; vi[n] = ci; vj[n] = cj; ++n;
        }
    }
}

// One of those cells: its bed from the corrected vertices and the conservative w / Hnpsi
// (cells of tiles that are not active are skipped; the reference updates its intermediate
// copy of a ghost tile there, which only the last hydraulic RHS of the step would read).
// Split in two so a warp can load the cell's step-start data (which the walk never
// changes) while another lane is still correcting the vertices.
// (The FP32 form loads the step-start Hn gam, clamped, and Hnpsi gam from the attempt's
// cache into hg / pg instead of the step-start w, Hnpsi, b0 and slopes.)
struct RedistCell {
    int ct, ci, cj;
    bool on;
    double b0n, b00, bt0, bx0, by0, w0, p0, hg, pg;
};
template <bool PLAIN>
__device__ __forceinline__ void redist_cell_load(const DevParams& P, const DevArrays& A, int qa, int tcur, int tnew, int ct, int ci,
                                                 int cj, RedistCell& r) {
    r.ct = ct; r.ci = ci; r.cj = cj;
    r.on = ct >= 0 && A.kind[ct] == SLOT_ACTIVE;
    if (!r.on) return;
    int SC = P.nX * P.nY;
    size_t cc = (size_t)cj * P.nX + ci;
    const double *C0 = A.CT[tcur], *C3 = A.CT[tnew];
    r.b0n = C3[mp(ct, 4, 0, SC) + cc];
    if (PLAIN) {
        const double* Z = A.M0 + mp(ct, 3, 0, SC) + cc;
        r.bt0 = C0[mp(ct, 4, 1, SC) + cc];
        r.hg = Z[0] < 0.0 ? 0.0 : Z[(size_t)SC];
        r.pg = Z[2 * (size_t)SC];
        return;
    }
    r.b00 = C0[mp(ct, 4, 0, SC) + cc];
    r.bt0 = C0[mp(ct, 4, 1, SC) + cc];
    r.bx0 = C0[mp(ct, 4, 2, SC) + cc];
    r.by0 = C0[mp(ct, 4, 3, SC) + cc];
    r.w0 = A.Q[qa][mp(ct, 4, 0, SC) + cc];
    r.p0 = A.Q[qa][mp(ct, 4, 3, SC) + cc];
}
template <bool PLAIN>
__device__ __forceinline__ void redist_cell_apply(const DevParams& P, const DevArrays& A, int tcur, int tnew, const RedistCell& r) {
    if (!r.on) return;
    int SC = P.nX * P.nY;
    size_t cc = (size_t)r.cj * P.nX + r.ci;
    if (PLAIN) {
        // the FP32 form's cell bed (as m_cells: static b0 parts from the cache, bt terms
        // summed plainly) and its w / Hnpsi update with 1/gamma from an FP32-seeded Newton step
        int nX = P.nX, SV = (nX + 1) * (P.nY + 1);
        const double* bt = A.BV[tnew] + mp(r.ct, 2, 1, SV);
        int v00 = r.cj * (nX + 1) + r.ci, v10 = v00 + 1, v01 = v00 + (nX + 1), v11 = v01 + 1;
        const double* B = A.B0S + mp(r.ct, 2, 0, SC) + cc;
        double btc = 0.25 * ((bt[v00] + bt[v10]) + (bt[v01] + bt[v11]));
        double dbx = B[0] + P.hdxR * ((bt[v10] - bt[v00]) + (bt[v11] - bt[v01]));
        double dby = B[(size_t)SC] + P.hdyR * ((bt[v01] - bt[v00]) + (bt[v11] - bt[v10]));
        A.CT[tnew][mp(r.ct, 4, 1, SC) + cc] = btc;
        A.CT[tnew][mp(r.ct, 4, 2, SC) + cc] = dbx;
        A.CT[tnew][mp(r.ct, 4, 3, SC) + cc] = dby;
        double dbc = btc - r.bt0;
        double ign = 1.0;
        if (P.geo) ign = rsqrt_nr(1.0 + (dbx * dbx + dby * dby));
        A.MS[mp(r.ct, 5, 0, SC) + cc] = (r.b0n + btc) + (r.hg - dbc) * (ign * ign);
        A.MS[mp(r.ct, 5, 1, SC) + cc] = (r.pg - (1.0 - P.BedPorosity) * dbc) * ign;
        return;
    }
    double c3[3];
    cell_topo_ij(P, A, tnew, r.ct, r.ci, r.cj, c3);
    double dbc = c3[0] - r.bt0;
    double go = gam_of(P.geo, r.bx0, r.by0);
    double gn = gam_of(P.geo, c3[1], c3[2]);
    double Hno = compute_hn(r.w0, r.b00, r.bt0, go);
    if (Hno < 0.0) Hno = 0.0;
    double w = c3[0];
    w = w + (Hno * go / gn - dbc / gn) / gn;
    w = w + r.b0n;
    A.MS[mp(r.ct, 5, 0, SC) + cc] = w;
    A.MS[mp(r.ct, 5, 1, SC) + cc] = r.p0 * go / gn - (1.0 - P.BedPorosity) * dbc / gn;
}
template <bool PLAIN>
__device__ __forceinline__ void redist_cell(const DevParams& P, const DevArrays& A, int qa, int tcur, int tnew, int ct, int ci,
                                            int cj) {
    RedistCell r;
    redist_cell_load<PLAIN>(P, A, qa, tcur, tnew, ct, ci, cj, r);
    redist_cell_apply<PLAIN>(P, A, tcur, tnew, r);
}

// RedistributeGrid (src/Redistribute.f90:203-244) over the ordered candidate list, run as
// dependency waves.  Candidate q touches the vertices of its own cell and the cell data of
// its 3 x 3 neighbourhood, and reads the vertices of that neighbourhood, so two candidates
// can only interact when their cells are within 2 cells of each other (Chebyshev distance,
// across tile seams).  The host puts each candidate in wave 1 + the largest wave of the
// earlier candidates it can interact with; inside a wave no two candidates interact, and
// every interacting pair keeps the list order, so the result equals the serial walk.
// One CTA walks the waves with a barrier between them (__syncthreads makes the global
// writes of a wave visible to the whole CTA).  A cell with no depositional vertex sets
// flags[0]; the remaining waves are then skipped, as the serial walk stops there.
template <bool PLAIN>
__device__ __forceinline__ void m_redist(const DevParams& P, const DevArrays& A, const int* __restrict__ list_slot,
                                         const int* __restrict__ list_cell, const int* __restrict__ wave_off, int nwaves,
                                         int qa, int tcur, int tnew, int* flags) {
    // One warp per candidate: lane 0 runs the excess test and the vertex correction, then
    // lanes 0..8 update the nine cells (distinct cells, no interaction between them).
    __shared__ int failed;
    if (threadIdx.x == 0) failed = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int wv = 0; wv < nwaves; ++wv) {
        for (int q = wave_off[wv] + warp; q < wave_off[wv + 1]; q += nwarps) {
            int s = list_slot[q], c = list_cell[q];
            int i = c % P.nX, j = c / P.nX;
            int go = 0;
            if (lane == 0) {
                double ex, dBt, psiold, Ho, Hn;
                excess_deposition<PLAIN>(P, A, s, c, qa, tcur, tnew, ex, dBt, psiold, Ho, Hn);
                if (ex > kEPS) {
                    if (redistribute_cell<PLAIN>(P, A, qa, tcur, tnew, s, i, j, ex)) go = 1;
                    else failed = 1;
                }
            }
            go = __shfl_sync(0xffffffffu, go, 0);
            __syncwarp();
            if (go) {
                int vt[9], vi[9], vj[9];
                redist_cells_of(P, A, s, i, j, vt, vi, vj);
                if (lane < 9) redist_cell<PLAIN>(P, A, qa, tcur, tnew, vt[lane], vi[lane], vj[lane]);
            }
            __syncwarp();
        }
        __syncthreads();
        if (failed) {
            if (threadIdx.x == 0) atomicOr(flags, 1);
            return;
        }
    }
}

// The M result becomes the input of the second hydraulic step: w and Hnpsi from the stage
// state, momenta unchanged.
__device__ __forceinline__ void m_finish(const DevParams& P, const DevArrays& A, int s, int item_, int qa) {
    int SC = P.nX * P.nY;
    if (item_ < SC) {
        int c = item_;
        A.Q[qa][mp(s, 4, 0, SC) + c] = A.MS[mp(s, 5, 0, SC) + c];
        A.Q[qa][mp(s, 4, 3, SC) + c] = A.MS[mp(s, 5, 1, SC) + c];
    }
}

// ---- single-simulation kernels: one thread per cell / vertex, `per` CTAs per listed tile ----
#define KG_TILE_ITEMS(NITEMS)                               \
    int per_ = ((NITEMS) + 255) / 256;                      \
    int pos = blockIdx.x / per_;                            \
    int s = slots[pos];                                     \
    int item_ = (blockIdx.x % per_) * 256 + threadIdx.x;    \
    (void)pos;

// ctl_flags[0..1]: the M refine flag and the candidate count, zeroed here for k_m_check.
template <bool PLAIN, bool ALT = false>
__global__ void __launch_bounds__(256) k_m_init(DevArrays A, const int* __restrict__ slots, int qa, int tcur, int tnew,
                                                int* ctl_flags) {
    kg_dep_wait();
    if (blockIdx.x == 0 && threadIdx.x < 2) ctl_flags[threadIdx.x] = 0;
    KG_TILE_ITEMS((cP.nX + 1) * (cP.nY + 1))
    m_init<PLAIN, ALT>(cP, cP32, A, s, item_, qa, tcur, tnew);
}
template <class R>
__global__ void __launch_bounds__(256) k_m_emd(DevArrays A, const int* __restrict__ slots, int tnew) {
    kg_dep_wait();
    KG_TILE_ITEMS(cP.nX * cP.nY)
    m_emd<R>(cP, cP32, A, s, item_, tnew);
}
template <bool PLAIN>
// dtp: when set, the M time step is twice the hydraulic dt the device computed (k_dt), for
// an M queued before the host has read that dt back.
__global__ void __launch_bounds__(256) k_m_bt(DevArrays A, const int* __restrict__ slots, int tcur, int tnew, int stage, double dt,
                                              const double* __restrict__ dtp) {
    kg_dep_wait();
    KG_TILE_ITEMS((cP.nX + 1) * (cP.nY + 1))
    m_bt<PLAIN>(cP, A, s, item_, tcur, tnew, stage, dtp ? 2.0 * dtp[0] : dt);
}
template <bool PLAIN>
__global__ void __launch_bounds__(256) k_m_cells(DevArrays A, const int* __restrict__ slots, int qa, int tcur, int tnew) {
    kg_dep_wait();
    KG_TILE_ITEMS(cP.nX * cP.nY)
    m_cells<PLAIN>(cP, cP32, A, s, item_, qa, tcur, tnew);
}
template <bool PLAIN>
__global__ void __launch_bounds__(256) k_m_check(DevArrays A, const int* __restrict__ slots, int qa, int tcur, int tnew, int* flags,
                                                 unsigned long long* cand_key, double* cand_ex, int* ncand, int cand_cap) {
    kg_dep_wait();
    KG_TILE_ITEMS(cP.nX * cP.nY)
    m_check<PLAIN>(cP, A, s, item_, pos, qa, tcur, tnew, flags, cand_key, cand_ex, ncand, cand_cap);
}
template <bool PLAIN>
__global__ void __launch_bounds__(REDIST_THREADS) k_m_redist(DevArrays A, const int* __restrict__ list_slot,
                                                             const int* __restrict__ list_cell,
                                                             const int* __restrict__ wave_off, int nwaves, int qa, int tcur,
                                                             int tnew, int* flags) {
    kg_dep_wait();
    m_redist<PLAIN>(cP, A, list_slot, list_cell, wave_off, nwaves, qa, tcur, tnew, flags);
}
// One wave of the ordered walk, one 32-thread CTA per listed cell, so the wave's FP64 work
// spreads over every SM (an SM has 2 FP64 lanes per clock).  A wave does nothing once an
// earlier wave found a cell without a depositional vertex (the serial walk stops there).
template <bool PLAIN>
__global__ void __launch_bounds__(32) k_m_redist_wave(DevArrays A, const int* __restrict__ list_slot,
                                                      const int* __restrict__ list_cell, int qa, int tcur, int tnew,
                                                      int* flags) {
    kg_dep_wait();
    const int lane = threadIdx.x;
    // The failure flag and the list entry are independent loads, issued together.
    int failed = *(volatile int*)flags;
    int s = list_slot[blockIdx.x], c = list_cell[blockIdx.x];
    if (failed != 0) return;
    int i = c % cP.nX, j = c / cP.nX;
    // Lanes 1..9 find their neighbour cell and load its step-start data while lane 0 runs
    // the excess test and the vertex correction.
    RedistCell r;
    r.on = false;
    if (lane >= 1 && lane <= 9) {
        int vt[9], vi[9], vj[9];
        redist_cells_of(cP, A, s, i, j, vt, vi, vj);
        int mt = -1, mi = 0, mj = 0;
#pragma unroll
        for (int k = 0; k < 9; ++k)
            if (k == lane - 1) { mt = vt[k]; mi = vi[k]; mj = vj[k]; }
        redist_cell_load<PLAIN>(cP, A, qa, tcur, tnew, mt, mi, mj, r);
    }
    int go = 0;
    if (lane == 0) {
        double ex, dBt, psiold, Ho, Hn;
        excess_deposition<PLAIN>(cP, A, s, c, qa, tcur, tnew, ex, dBt, psiold, Ho, Hn);
        if (ex > kEPS) {
            if (redistribute_cell<PLAIN>(cP, A, qa, tcur, tnew, s, i, j, ex)) go = 1;
            else atomicOr(flags, 1);
        }
    }
    go = __shfl_sync(0xffffffffu, go, 0);
    __syncwarp();  // lane 0's vertex writes are visible to the other lanes after this
    if (go) redist_cell_apply<PLAIN>(cP, A, tcur, tnew, r);
}

template <bool PLAIN>
__device__ __forceinline__ void m_close(const DevParams& P, const DevArrays& A, int s, int k, int qa, int tnew) {
    face_topo<PLAIN>(P, A, s, k, tnew);
    face_bI(P, A, s, k, tnew);
    m_finish(P, A, s, k, qa);
    if (PLAIN) topo32(P, A, s, k, tnew);
}
template <bool PLAIN>
__global__ void __launch_bounds__(256) k_m_close(DevArrays A, const int* __restrict__ slots, int qa, int tnew, int per) {
    kg_dep_wait();
    m_close<PLAIN>(cP, A, slots[blockIdx.x / per], (blockIdx.x % per) * 256 + threadIdx.x, qa, tnew);
}

// ---- FP32 form: one launch per M stage (single simulation) ----
// k_m_stage32<STAGE> runs a whole stage of M for one MSB x MSB block of cells of an active
// tile, in place of the k_m_emd / k_m_bt / k_m_cells launches:
//   0. the dry test of every cell within two cells of the block (the stage depth below the
//      height threshold; ghost tiles from their static data, tiles never allocated dry);
//   1. E - D (as m_emd) and the slopes of the block's cells and of the ring of cells around
//      it, whichever of the eight neighbouring tiles they lie in (zero E - D outside active
//      tiles, as the vertex source reads it);
//   2. the vertex source and the clamped bed update (as m_bt) of the block's
//      (MSB + 1)^2 vertices from those values in shared memory;
//   3. the cell bed, the w / Hnpsi update and the stage variables (cell32_update) of the
//      block's own cells from the new vertices in shared memory;
//   4. after the third stage, the refinement tests (m_check) of its own cells.
// The shared helpers form every value with the same operations on the same operands, so the
// stages equal the three per-item launches (which the batched engine runs) bit for bit.
// Each block reads the stage variables of cells that other blocks write in the same launch,
// so those alternate between two copies from stage to stage: the stage depth (MS plane 2 /
// 3), the six float stage planes (MF_HN.. / MF_AHN..) and the vertex bt (BV[tnew] plane 1 /
// BVA).  m_init<true, true> fills the second copies; stages 1 and 3 read the second copies
// and write the first, stage 2 the reverse, so the M result ends in the first copies, where
// the tests, the redistribution walk and the closing launch read it (the vertex bt: stage 1
// writes BV[tnew], stage 2 BVA, stage 3 BV[tnew]).  A cell whose bed did not change carries
// its stage variables forward into the copy being written.
constexpr int MSB = 16;
struct MStageSmem {
    unsigned char dry[MSB + 4][MSB + 4];
    float ef[MSB + 2][MSB + 2], xf[MSB + 2][MSB + 2], yf[MSB + 2][MSB + 2];
    double bt[MSB + 1][MSB + 1], bt0[MSB + 1][MSB + 1];
};

// Slot (-1: a tile never allocated) and cell index of tile-local cell (i, j) of tile s, which
// may lie in one of the eight tiles around s: the column's tile (W / E) first, then its south
// or north neighbour, as the vertex source and the redistribution walk reach corner tiles.
// |i| and |j| stay within one tile of s (tiles of at least 2 x 2 cells).
__device__ __forceinline__ int stage_cell_slot(const DevArrays& A, int s, int sW, int sE, int nX, int nY, int i, int j, int& c) {
    int col = s;
    if (i < 0) { col = sW; i += nX; }
    else if (i >= nX) { col = sE; i -= nX; }
    int t = col;
    if (j < 0) { t = col < 0 ? -1 : A.nbr[col * 8 + NB_S]; j += nY; }
    else if (j >= nY) { t = col < 0 ? -1 : A.nbr[col * 8 + NB_N]; j -= nY; }
    c = j * nX + i;
    return t;
}

template <int STAGE>
__global__ void __launch_bounds__(256) k_m_stage32(DevArrays A, const int* __restrict__ slots, int nbt, int qa, int tcur, int tnew,
                                                   double dt_m, const double* __restrict__ dtp, int* flags,
                                                   unsigned long long* cand_key, double* cand_ex, int* ncand, int cand_cap) {
    kg_dep_wait();
    __shared__ MStageSmem sm;
    const DevParams& P = cP;
    const int nX = P.nX, nY = P.nY, SC = nX * nY, SV = (nX + 1) * (nY + 1);
    const int pos = blockIdx.x / nbt, blk = blockIdx.x % nbt, nbx = (nX + MSB - 1) / MSB;
    const int x0 = (blk % nbx) * MSB, y0 = (blk / nbx) * MSB;
    const int bx = min(MSB, nX - x0), by = min(MSB, nY - y0);
    const int s = slots[pos];
    const int sW = A.nbr[s * 8 + NB_W], sE = A.nbr[s * 8 + NB_E];
    const int tid = threadIdx.x;
    // stages 1 and 3 read the second copies and write the first; stage 2 the reverse
    constexpr bool RD_ALT = STAGE != 2;
    constexpr int hn_rd = RD_ALT ? 3 : 2, hn_wr = RD_ALT ? 2 : 3;
    constexpr int mf_rd = RD_ALT ? MF_ALT : 0, mf_wr = RD_ALT ? 0 : MF_ALT;
    double* bt_rd = STAGE == 2 ? A.BV[tnew] + mp(s, 2, 1, SV) : A.BVA + (size_t)s * SV;
    double* bt_wr = STAGE == 2 ? A.BVA + (size_t)s * SV : A.BV[tnew] + mp(s, 2, 1, SV);

    // 0. dry flags of the (bx + 4) x (by + 4) box around the block
    for (int k = tid; k < (bx + 4) * (by + 4); k += blockDim.x) {
        const int cx = k % (bx + 4) - 2, cy = k / (bx + 4) - 2;
        int c;
        const int t = stage_cell_slot(A, s, sW, sE, nX, nY, x0 + cx, y0 + cy, c);
        bool dry = true;
        if (t >= 0) dry = below_pos(A.kind[t] == SLOT_GHOST ? A.G9[mp(t, 9, 4, SC) + c] : A.MS[mp(t, 5, hn_rd, SC) + c], P.hThr);
        sm.dry[cy + 2][cx + 2] = dry;
    }
    __syncthreads();
    // 1. E - D and slopes of the block's cells and the ring around them
    for (int k = tid; k < (bx + 2) * (by + 2); k += blockDim.x) {
        const int cx = k % (bx + 2) - 1, cy = k / (bx + 2) - 1;
        int c;
        const int t = stage_cell_slot(A, s, sW, sE, nX, nY, x0 + cx, y0 + cy, c);
        float ef = 0.f, xf = 0.f, yf = 0.f;
        if (t >= 0 && A.kind[t] == SLOT_ACTIVE) {
            xf = mfp(A, t, MF_BX + mf_rd, SC)[c];
            yf = mfp(A, t, MF_BY + mf_rd, SC)[c];
            const int X = cx + 2, Y = cy + 2;
            if (!(sm.dry[Y][X] || sm.dry[Y][X - 1] || sm.dry[Y][X + 1] || sm.dry[Y - 1][X] || sm.dry[Y + 1][X]))
                ef = emd32(P, cP32, A, t, c, SC, mf_rd, xf, yf);
        } else if (t >= 0) {
            xf = A.TF[tcur][mp(t, 6, 1, SC) + c];
            yf = A.TF[tcur][mp(t, 6, 2, SC) + c];
        }
        sm.ef[cy + 1][cx + 1] = ef;
        sm.xf[cy + 1][cx + 1] = xf;
        sm.yf[cy + 1][cx + 1] = yf;
    }
    __syncthreads();
    // 2. the block's vertices: cells south-west, north-west, south-east, north-east of each
    const double dt = dtp ? 2.0 * dtp[0] : dt_m;
    for (int k = tid; k < (bx + 1) * (by + 1); k += blockDim.x) {
        const int a = k % (bx + 1), b = k / (bx + 1);
        const float ef[4] = {sm.ef[b][a], sm.ef[b + 1][a], sm.ef[b][a + 1], sm.ef[b + 1][a + 1]};
        const float xf[4] = {sm.xf[b][a], sm.xf[b + 1][a], sm.xf[b][a + 1], sm.xf[b + 1][a + 1]};
        const float yf[4] = {sm.yf[b][a], sm.yf[b + 1][a], sm.yf[b][a + 1], sm.yf[b + 1][a + 1]};
        const int v = (y0 + b) * (nX + 1) + (x0 + a);
        const double bt0 = A.BV[tcur][mp(s, 2, 1, SV) + v];
        const double btp = STAGE == 1 ? bt0 : bt_rd[v];
        const double nb = bt32_stage(P, STAGE, bt0, btp, dt, ddt32_vertex(P, ef, xf, yf));
        bt_wr[v] = nb;
        sm.bt[b][a] = nb;
        sm.bt0[b][a] = bt0;
    }
    __syncthreads();
    // 3. the block's own cells
    if (tid < bx * by) {
        const int cx = tid % bx, cy = tid / bx, c = (y0 + cy) * nX + (x0 + cx);
        const double b00 = sm.bt[cy][cx], b10 = sm.bt[cy][cx + 1], b01 = sm.bt[cy + 1][cx], b11 = sm.bt[cy + 1][cx + 1];
        const double *C0 = A.CT[tcur], *C3 = A.CT[tnew];
        if (same_bits(b00, sm.bt0[cy][cx]) && same_bits(b10, sm.bt0[cy][cx + 1]) && same_bits(b01, sm.bt0[cy + 1][cx]) &&
            same_bits(b11, sm.bt0[cy + 1][cx + 1]) && same_bits(C3[mp(s, 4, 1, SC) + c], C0[mp(s, 4, 1, SC) + c]) &&
            same_bits(C3[mp(s, 4, 2, SC) + c], C0[mp(s, 4, 2, SC) + c]) && same_bits(C3[mp(s, 4, 3, SC) + c], C0[mp(s, 4, 3, SC) + c])) {
            // bed unchanged: the stage state carries forward
            A.MS[mp(s, 5, hn_wr, SC) + c] = A.MS[mp(s, 5, hn_rd, SC) + c];
#pragma unroll
            for (int f = MF_HN; f <= MF_BY; ++f) mfp(A, s, f + mf_wr, SC)[c] = mfp(A, s, f + mf_rd, SC)[c];
        } else {
            cell32_update(P, cP32, A, s, c, tcur, tnew, b00, b10, b01, b11, hn_wr, mf_wr);
        }
        // 4. the refinement tests after the last stage (the cell's own values, written above)
        if (STAGE == 3) m_check<true>(P, A, s, c, pos, qa, tcur, tnew, flags, cand_key, cand_ex, ncand, cand_cap);
    }
}

// Blocks of the fused stage per tile; 0 when the tiles are too small for its two-cell halo
// (the three per-item launches run then).
int m_stage32_blocks(int nX, int nY) {
    if (nX < 2 || nY < 2) return 0;
    return ((nX + MSB - 1) / MSB) * ((nY + MSB - 1) / MSB);
}

// ---- host launchers (cells/verts: items per tile) ----
static inline int per_of(int items) { return (items + 255) / 256; }

cudaError_t launch_m_init(const DevArrays& A, const int* d_slots, int n, int verts, int qa, int tcur, int tnew, int* ctl_flags,
                          bool fp32, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (fp32) KG_TRY_LAUNCH(kg_launch(k_m_init<true>, n * per_of(verts), 256, 0, st, A, d_slots, qa, tcur, tnew, ctl_flags));
    else KG_TRY_LAUNCH(kg_launch(k_m_init<false>, n * per_of(verts), 256, 0, st, A, d_slots, qa, tcur, tnew, ctl_flags));
    return cudaGetLastError();
}
// The FP32 form's fused M attempt up to its tests: init into the second copies of the stage
// planes, then one k_m_stage32 launch per stage (the third runs the tests).
cudaError_t launch_m_fused32(const DevArrays& A, const int* d_slots, int n, int nX, int nY, int qa, int tcur, int tnew,
                             double dt_m, const double* dtp, int* ctl_flags, unsigned long long* keys, double* ex, int* ncand,
                             int cap, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int nbt = m_stage32_blocks(nX, nY);
    if (nbt <= 0) return cudaErrorInvalidValue;
    KG_TRY_LAUNCH(kg_launch(k_m_init<true, true>, n * per_of((nX + 1) * (nY + 1)), 256, 0, st, A, d_slots, qa, tcur, tnew, ctl_flags));
    KG_TRY_LAUNCH(kg_launch(k_m_stage32<1>, n * nbt, 256, 0, st, A, d_slots, nbt, qa, tcur, tnew, dt_m, dtp, ctl_flags, keys, ex, ncand, cap));
    KG_TRY_LAUNCH(kg_launch(k_m_stage32<2>, n * nbt, 256, 0, st, A, d_slots, nbt, qa, tcur, tnew, dt_m, dtp, ctl_flags, keys, ex, ncand, cap));
    KG_TRY_LAUNCH(kg_launch(k_m_stage32<3>, n * nbt, 256, 0, st, A, d_slots, nbt, qa, tcur, tnew, dt_m, dtp, ctl_flags, keys, ex, ncand, cap));
    return cudaGetLastError();
}
cudaError_t launch_m_emd(const DevArrays& A, const int* d_slots, int n, int cells, int tnew, bool fp32, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (fp32) KG_TRY_LAUNCH(kg_launch(k_m_emd<float>, n * per_of(cells), 256, 0, st, A, d_slots, tnew));
    else KG_TRY_LAUNCH(kg_launch(k_m_emd<double>, n * per_of(cells), 256, 0, st, A, d_slots, tnew));
    return cudaGetLastError();
}
cudaError_t launch_m_bt(const DevArrays& A, const int* d_slots, int n, int verts, int tcur, int tnew, int stage, double dt,
                        const double* dtp, bool fp32, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (fp32) KG_TRY_LAUNCH(kg_launch(k_m_bt<true>, n * per_of(verts), 256, 0, st, A, d_slots, tcur, tnew, stage, dt, dtp));
    else KG_TRY_LAUNCH(kg_launch(k_m_bt<false>, n * per_of(verts), 256, 0, st, A, d_slots, tcur, tnew, stage, dt, dtp));
    return cudaGetLastError();
}
cudaError_t launch_m_cells(const DevArrays& A, const int* d_slots, int n, int cells, int qa, int tcur, int tnew, bool fp32,
                           cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (fp32) KG_TRY_LAUNCH(kg_launch(k_m_cells<true>, n * per_of(cells), 256, 0, st, A, d_slots, qa, tcur, tnew));
    else KG_TRY_LAUNCH(kg_launch(k_m_cells<false>, n * per_of(cells), 256, 0, st, A, d_slots, qa, tcur, tnew));
    return cudaGetLastError();
}
cudaError_t launch_m_check(const DevArrays& A, const int* d_slots, int n, int cells, int qa, int tcur, int tnew, int* flags,
                           unsigned long long* keys, double* ex, int* ncand, int cap, bool fp32, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (fp32) KG_TRY_LAUNCH(kg_launch(k_m_check<true>, n * per_of(cells), 256, 0, st, A, d_slots, qa, tcur, tnew, flags, keys, ex, ncand, cap));
    else KG_TRY_LAUNCH(kg_launch(k_m_check<false>, n * per_of(cells), 256, 0, st, A, d_slots, qa, tcur, tnew, flags, keys, ex, ncand, cap));
    return cudaGetLastError();
}
// hwoff: the wave offsets on the host (one launch per wave while the waves are few).
cudaError_t launch_m_redist(const DevArrays& A, const int* ls, const int* lc, const int* woff, const int* hwoff, int nwaves,
                            int qa, int tcur, int tnew, int* flags, bool fp32, cudaStream_t st) {
    if (nwaves == 0) return cudaSuccess;
    if (nwaves > KG_REDIST_WAVE_MAX) {
        if (fp32) KG_TRY_LAUNCH(kg_launch(k_m_redist<true>, 1, REDIST_THREADS, 0, st, A, ls, lc, woff, nwaves, qa, tcur, tnew, flags));
        else KG_TRY_LAUNCH(kg_launch(k_m_redist<false>, 1, REDIST_THREADS, 0, st, A, ls, lc, woff, nwaves, qa, tcur, tnew, flags));
        return cudaGetLastError();
    }
    for (int w = 0; w < nwaves; ++w) {
        int n = hwoff[w + 1] - hwoff[w];
        if (n <= 0) continue;
        if (fp32) KG_TRY_LAUNCH(kg_launch(k_m_redist_wave<true>, n, 32, 0, st, A, ls + hwoff[w], lc + hwoff[w], qa, tcur, tnew, flags));
        else KG_TRY_LAUNCH(kg_launch(k_m_redist_wave<false>, n, 32, 0, st, A, ls + hwoff[w], lc + hwoff[w], qa, tcur, tnew, flags));
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
// The end of an M attempt in one launch: the interfacial topography of the new bed
// (face_topo, face_bI), the M result into state qa (m_finish) and, in the FP32 form, the
// factor cache of the new topography set for the listed tiles (topo32).  Every part works
// on item k of the tile (face k, cell k) and reads only data written before the launch or
// by the same thread, so the four kernels fuse without changing a result.
cudaError_t launch_m_close(const DevArrays& A, const int* d_slots, int n, int nX, int nY, int qa, int tnew, bool fp32,
                           cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int per = per_of((nX + 1) * (nY + 1));
    if (fp32) KG_TRY_LAUNCH(kg_launch(k_m_close<true>, n * per, 256, 0, st, A, d_slots, qa, tnew, per));
    else KG_TRY_LAUNCH(kg_launch(k_m_close<false>, n * per, 256, 0, st, A, d_slots, qa, tnew, per));
    return cudaGetLastError();
}

}  // namespace kg
