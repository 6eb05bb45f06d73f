// kg_tiles.cu -- tile set-up, activation and accounting kernels.
//
//   k_cell_topo     ComputeCellCentredTopographicData   src/MorphodynamicRHS.f90:308-366
//   k_face_bI       InterpolateB at every face           src/HydraulicRHS.f90:741-753
//   k_face_topo     ComputeInterfacialTopographicData    src/MorphodynamicRHS.f90:419-540
//   k_ghost_bc      UpdateGhostTileBCs                   src/UpdateTiles.f90:571-664
//   k_ghost_edges   ReconstructwAtEdges                  src/UpdateTiles.f90:669-750
//   k_activate      ActivateTile's w = b, bt = 0         src/UpdateTiles.f90:342-370
//   k_act_flags     the per-direction tests of CheckIfNearBoundaries
//                                                        src/TimeStepper.f90:924-1150
//   k_volume        CalculateVolume's four compensated sums, in the reference's order
//                                                        src/Output.f90:617-737
#include <cuda_runtime.h>
#include "kg_engine.cuh"

namespace kg {

// cP (the run settings in constant memory) is defined in kg_hydro.cu; both files are
// compiled as one translation unit through kg_lib.cu.

__device__ __forceinline__ size_t pl(int slot, int nf, int f, int npl) { return ((size_t)slot * nf + f) * (size_t)npl; }

// One CTA per listed slot.
__global__ void k_cell_topo(DevArrays A, const int* __restrict__ slots, int ts) {
    const DevParams& P = cP;
    int s = slots[blockIdx.x];
    int nX = P.nX, nY = P.nY, SC = nX * nY, SV = (nX + 1) * (nY + 1);
    const double* b0 = A.BV[ts] + pl(s, 2, 0, SV);
    const double* bt = A.BV[ts] + pl(s, 2, 1, SV);
    double* CT = A.CT[ts];
    for (int c = threadIdx.x; c < SC; c += blockDim.x) {
        int i = c % nX, j = c / nX;
        int v00 = j * (nX + 1) + i, v10 = v00 + 1, v01 = v00 + (nX + 1), v11 = v01 + 1;
        double b0c = 0.25 * kahan4(b0[v00], b0[v10], b0[v01], b0[v11]);
        double btc = 0.25 * kahan4(bt[v00], bt[v10], bt[v01], bt[v11]);
        double ax[8] = {b0[v10], bt[v10], -b0[v00], -bt[v00], b0[v11], bt[v11], -b0[v01], -bt[v01]};
        double ay[8] = {b0[v01], bt[v01], -b0[v00], -bt[v00], b0[v11], bt[v11], -b0[v10], -bt[v10]};
        CT[pl(s, 4, 0, SC) + c] = b0c;
        CT[pl(s, 4, 1, SC) + c] = btc;
        CT[pl(s, 4, 2, SC) + c] = 0.5 * P.dxR * kahan8(ax);
        CT[pl(s, 4, 3, SC) + c] = 0.5 * P.dyR * kahan8(ay);
        // The static b0 parts of the slopes, which the FP32 form's M stages add to the bt parts.
        A.B0S[pl(s, 2, 0, SC) + c] = P.hdxR * ((b0[v10] - b0[v00]) + (b0[v11] - b0[v01]));
        A.B0S[pl(s, 2, 1, SC) + c] = P.hdyR * ((b0[v01] - b0[v00]) + (b0[v11] - b0[v10]));
    }
}

// Per-tile kernels over the faces / cells of the listed tiles run `per` CTAs of 256
// threads per tile, one face (x and y) or cell per thread.
__device__ __forceinline__ void face_bI(const DevParams& P, const DevArrays& A, int s, int f, int ts) {
    int nX = P.nX, nY = P.nY, SV = (nX + 1) * (nY + 1), SFX = (nX + 1) * nY, SFY = nX * (nY + 1);
    const double* b0 = A.BV[ts] + pl(s, 2, 0, SV);
    const double* bt = A.BV[ts] + pl(s, 2, 1, SV);
    if (f < SFX) {
        int a = f % (nX + 1), j = f / (nX + 1);
        int v0 = j * (nX + 1) + a, v1 = v0 + (nX + 1);
        A.FX[ts][pl(s, 5, 4, SFX) + f] = interp_b(b0[v0], b0[v1], bt[v0], bt[v1]);
    }
    if (f < SFY) {
        int i = f % nX, a = f / nX;
        int v0 = a * (nX + 1) + i, v1 = v0 + 1;
        A.FY[ts][pl(s, 5, 4, SFY) + f] = interp_b(b0[v0], b0[v1], bt[v0], bt[v1]);
    }
}

// Face bt and slopes of one tile from its own vertices and the adjacent column/row of
// the W/E/S/N tiles' vertex copies.  PLAIN (the FP32 form) sums the vertex terms pairwise
// in FP64, differences first, instead of the reference's compensated sums.
template <bool PLAIN>
__device__ __forceinline__ void face_topo(const DevParams& P, const DevArrays& A, int s, int f, int ts) {
    int nX = P.nX, nY = P.nY, SV = (nX + 1) * (nY + 1), SFX = (nX + 1) * nY, SFY = nX * (nY + 1);
    int sW = A.nbr[s * 8 + NB_W], sE = A.nbr[s * 8 + NB_E], sS = A.nbr[s * 8 + NB_S], sN = A.nbr[s * 8 + NB_N];
    const double* BV = A.BV[ts];
    double* FXs = A.FX[ts];
    double* FYs = A.FY[ts];
    const double* b0 = BV + pl(s, 2, 0, SV);
    const double* bt = BV + pl(s, 2, 1, SV);
    const int V = nX + 1;
    if (f < SFX) {
        int a = f % (nX + 1), j = f / (nX + 1);  // vertex column a, rows j..j+1
        // d/dx from the vertex columns either side (the W/E tile's copy at the tile edge)
        const double *lb0 = b0, *lbt = bt, *rb0 = b0, *rbt = bt;
        int la = a - 1, ra = a + 1;
        if (a == 0) { lb0 = BV + pl(sW, 2, 0, SV); lbt = BV + pl(sW, 2, 1, SV); la = nX - 1; }
        if (a == nX) { rb0 = BV + pl(sE, 2, 0, SV); rbt = BV + pl(sE, 2, 1, SV); ra = 1; }
        int v0 = j * V + a, v1 = v0 + V;
        double btf = 0.5 * (bt[v0] + bt[v1]);
        double dbdx, dbdy;
        if (PLAIN) {
            dbdx = 0.25 * P.dxR * (((rb0[j * V + ra] - lb0[j * V + la]) + (rbt[j * V + ra] - lbt[j * V + la])) +
                                   ((rb0[(j + 1) * V + ra] - lb0[(j + 1) * V + la]) + (rbt[(j + 1) * V + ra] - lbt[(j + 1) * V + la])));
            dbdy = P.dyR * ((b0[v1] - b0[v0]) + (bt[v1] - bt[v0]));
        } else {
            double ax[8] = {rb0[j * V + ra], rbt[j * V + ra], rb0[(j + 1) * V + ra], rbt[(j + 1) * V + ra],
                            -lb0[j * V + la], -lbt[j * V + la], -lb0[(j + 1) * V + la], -lbt[(j + 1) * V + la]};
            dbdx = 0.25 * P.dxR * kahan8(ax);
            double ay[4] = {b0[v1], bt[v1], -b0[v0], -bt[v0]};
            dbdy = P.dyR * kahan4(ay[0], ay[1], ay[2], ay[3]);
        }
        FXs[pl(s, 5, 1, SFX) + f] = btf;
        FXs[pl(s, 5, 2, SFX) + f] = dbdx;
        FXs[pl(s, 5, 3, SFX) + f] = dbdy;
    }
    if (f < SFY) {
        int i = f % nX, a = f / nX;  // vertex row a, columns i..i+1
        int v0 = a * V + i, v1 = v0 + 1;
        double btf = 0.5 * (bt[v0] + bt[v1]);
        const double *db0 = b0, *dbt = bt, *ub0 = b0, *ubt = bt;
        int da = a - 1, ua = a + 1;
        if (a == 0) { db0 = BV + pl(sS, 2, 0, SV); dbt = BV + pl(sS, 2, 1, SV); da = nY - 1; }
        if (a == nY) { ub0 = BV + pl(sN, 2, 0, SV); ubt = BV + pl(sN, 2, 1, SV); ua = 1; }
        double dbdx, dbdy;
        if (PLAIN) {
            dbdx = P.dxR * ((b0[v1] - b0[v0]) + (bt[v1] - bt[v0]));
            dbdy = 0.25 * P.dyR * (((ub0[ua * V + i + 1] - db0[da * V + i + 1]) + (ubt[ua * V + i + 1] - dbt[da * V + i + 1])) +
                                   ((ub0[ua * V + i] - db0[da * V + i]) + (ubt[ua * V + i] - dbt[da * V + i])));
        } else {
            double axv[4] = {b0[v1], bt[v1], -b0[v0], -bt[v0]};
            dbdx = P.dxR * kahan4(axv[0], axv[1], axv[2], axv[3]);
            double ay[8] = {ub0[ua * V + i + 1], ubt[ua * V + i + 1], ub0[ua * V + i], ubt[ua * V + i],
                            -db0[da * V + i + 1], -dbt[da * V + i + 1], -db0[da * V + i], -dbt[da * V + i]};
            dbdy = 0.25 * P.dyR * kahan8(ay);
        }
        FYs[pl(s, 5, 1, SFY) + f] = btf;
        FYs[pl(s, 5, 2, SFY) + f] = dbdx;
        FYs[pl(s, 5, 3, SFY) + f] = dbdy;
    }
}

__global__ void __launch_bounds__(256) k_face_bI(DevArrays A, const int* __restrict__ slots, int ts, int per) {
    face_bI(cP, A, slots[blockIdx.x / per], (blockIdx.x % per) * 256 + threadIdx.x, ts);
}
template <bool PLAIN>
__global__ void __launch_bounds__(256) k_face_topo(DevArrays A, const int* __restrict__ slots, int ts, int per) {
    face_topo<PLAIN>(cP, A, slots[blockIdx.x / per], (blockIdx.x % per) * 256 + threadIdx.x, ts);
}

// mode 0: default data (w = b0, rho = rhow, rest 0; SetDefaultTileData); 2: a periodic
// domain-edge ghost, which SetDomainBoundaryData leaves as allocated (zeros, rho = rhow).
__global__ void k_ghost_bc(DevArrays A, int slot, int mode, int ts) {
    const DevParams& P = cP;
    int SC = P.nX * P.nY;
    double* G = A.G9 + pl(slot, 9, 0, SC);
    for (int c = threadIdx.x; c < SC; c += blockDim.x) {
        for (int f = 0; f < 8; ++f) G[f * (size_t)SC + c] = 0.0;
        G[8 * (size_t)SC + c] = P.rhow;
        if (mode == 0) G[c] = A.CT[ts][pl(slot, 4, 0, SC) + c];
    }
}

// Dirichlet data (SetDomainBoundaryData 'dirichlet', src/UpdateTiles.f90:614-638).
__global__ void k_ghost_dirichlet(DevArrays A, int slot, double Hnval, double uval, double vval, double psival, int ts) {
    const DevParams& P = cP;
    int SC = P.nX * P.nY;
    double* G = A.G9 + pl(slot, 9, 0, SC);
    double rho = density(P, psival);
    for (int c = threadIdx.x; c < SC; c += blockDim.x) {
        const double* CT = A.CT[ts];
        double b0 = CT[pl(slot, 4, 0, SC) + c], bt = CT[pl(slot, 4, 1, SC) + c];
        double dbx = CT[pl(slot, 4, 2, SC) + c], dby = CT[pl(slot, 4, 3, SC) + c];
        double hpval = Hnval / gam_of(P.geo, dbx, dby);
        double w = bt + hpval;
        w = w + b0;
        G[c] = w;
        G[1 * (size_t)SC + c] = rho * Hnval * uval;
        G[2 * (size_t)SC + c] = rho * Hnval * vval;
        G[3 * (size_t)SC + c] = Hnval * psival;
        G[4 * (size_t)SC + c] = Hnval;
        G[5 * (size_t)SC + c] = uval;
        G[6 * (size_t)SC + c] = vval;
        G[7 * (size_t)SC + c] = psival;
        G[8 * (size_t)SC + c] = rho;
    }
}

// ReconstructwAtEdges for one ghost slot; edge bit k set when that neighbour (W,E,S,N) is
// an active tile whose current w lives in Q[qcur].
__global__ void k_ghost_edges(DevArrays A, int slot, int mask, int qcur) {
    const DevParams& P = cP;
    int nX = P.nX, nY = P.nY, SC = nX * nY, nE = A.nE;
    const double* w = A.G9 + pl(slot, 9, 0, SC);
    double* GE = A.GE + pl(slot, GE_COUNT, 0, nE);
    const double* Qc = A.Q[qcur];
    int lim = P.limiter;
    double dx = P.dx, dy = P.dy;
    for (int k = threadIdx.x; k < nY; k += blockDim.x) {
        int j = k;
        if (mask & 1) {
            int nb = A.nbr[slot * 8 + NB_W];
            double uW = Qc[pl(nb, 4, 0, SC) + j * nX + nX - 1];
            double l = P.dxR * limiter(lim, w[j * nX + 1] - w[j * nX], w[j * nX] - uW);
            GE[GE_LX1 * nE + j] = l;
            GE[GE_PX1 * nE + j] = w[j * nX] - l * 0.5 * dx;
            GE[GE_MX2 * nE + j] = w[j * nX] + l * 0.5 * dx;
        }
        if (mask & 2) {
            int nb = A.nbr[slot * 8 + NB_E];
            double uE = Qc[pl(nb, 4, 0, SC) + j * nX + 0];
            double l = P.dxR * limiter(lim, uE - w[j * nX + nX - 1], w[j * nX + nX - 1] - w[j * nX + nX - 2]);
            GE[GE_LXN * nE + j] = l;
            GE[GE_PXN * nE + j] = w[j * nX + nX - 1] - l * 0.5 * dx;
            GE[GE_MXN1 * nE + j] = w[j * nX + nX - 1] + l * 0.5 * dx;
        }
    }
    for (int i = threadIdx.x; i < nX; i += blockDim.x) {
        if (mask & 4) {
            int nb = A.nbr[slot * 8 + NB_S];
            double uS = Qc[pl(nb, 4, 0, SC) + (nY - 1) * nX + i];
            double l = P.dyR * limiter(lim, w[nX + i] - w[i], w[i] - uS);
            GE[GE_LY1 * nE + i] = l;
            GE[GE_PY1 * nE + i] = w[i] - l * 0.5 * dy;
            GE[GE_MY2 * nE + i] = w[i] + l * 0.5 * dy;
        }
        if (mask & 8) {
            int nb = A.nbr[slot * 8 + NB_N];
            double uN = Qc[pl(nb, 4, 0, SC) + 0 * nX + i];
            double wt = w[(nY - 1) * nX + i], wb = w[(nY - 2) * nX + i];
            double l = P.dyR * limiter(lim, uN - wt, wt - wb);
            GE[GE_LYN * nE + i] = l;
            GE[GE_PYN * nE + i] = wt - l * 0.5 * dy;
            GE[GE_MYN1 * nE + i] = wt + l * 0.5 * dy;
        }
    }
}

// ActivateTile: w = cell b0, cell bt = 0, momenta and Hnpsi as the tile held them (zero).
__global__ void k_activate(DevArrays A, int slot, int qcur, int ts) {
    const DevParams& P = cP;
    int SC = P.nX * P.nY;
    for (int c = threadIdx.x; c < SC; c += blockDim.x) {
        double b0 = A.CT[ts][pl(slot, 4, 0, SC) + c];
        A.CT[ts][pl(slot, 4, 1, SC) + c] = 0.0;
        double* Q = A.Q[qcur];
        Q[pl(slot, 4, 0, SC) + c] = b0;
        Q[pl(slot, 4, 1, SC) + c] = 0.0;
        Q[pl(slot, 4, 2, SC) + c] = 0.0;
        Q[pl(slot, 4, 3, SC) + c] = 0.0;
        A.UV[pl(slot, 2, 0, SC) + c] = 0.0;
        A.UV[pl(slot, 2, 1, SC) + c] = 0.0;
        A.EMD[(size_t)slot * SC + c] = 0.0;
    }
}

__global__ void k_init_maxima(DevArrays A, int slot) {
    int SC = cP.nX * cP.nY;
    double* M = A.MX + pl(slot, 11, 0, SC);
    for (int c = threadIdx.x; c < SC; c += blockDim.x) {
        for (int f = 0; f < 10; ++f) M[f * (size_t)SC + c] = 0.0;
        M[10 * (size_t)SC + c] = -1.0;
    }
}

// Edge-band tests of NearNorth/South/East/WestBoundary (src/TimeStepper.f90:924-1150):
// bit 0 N, 1 S, 2 E, 3 W of one thread's cell in 256-cell chunk `chunk` of slot s.
// hn_over (optional) replaces the depth computed from w (used for the first check after
// the sources have set the depth field directly).
__device__ __forceinline__ int act_bits(const DevParams& P, const DevArrays& A, int s, int qcur, int ts,
                                        const double* __restrict__ hn_over, int chunk) {
    int nX = P.nX, nY = P.nY, SC = nX * nY, TB = P.TileBuffer;
    const double* Q = A.Q[qcur];
    int f = 0;
    int c = chunk * 256 + threadIdx.x;
    if (c < SC) {
        int i = c % nX, j = c / nX;
        double Hn;
        if (hn_over) {
            Hn = hn_over[(size_t)s * SC + c];
        } else {
            const double* CT = A.CT[ts];
            double b0 = CT[pl(s, 4, 0, SC) + c], bt = CT[pl(s, 4, 1, SC) + c];
            double gam = gam_of(P.geo, CT[pl(s, 4, 2, SC) + c], CT[pl(s, 4, 3, SC) + c]);
            Hn = compute_hn(Q[pl(s, 4, 0, SC) + c], b0, bt, gam);
            if (Hn < 0.0) Hn = 0.0;
        }
        if (Hn > P.hThr) {
            int jj = j + 1, ii = i + 1;
            if (jj > nY - TB) f |= 1;
            if (jj <= TB) f |= 2;
            if (ii > nX - TB) f |= 4;
            if (ii <= TB) f |= 8;
        }
    }
    // The reference's scans start from ydist = 0 (N, E) or nY/nX (S, W), so a buffer
    // wider than the tile triggers without any wet cell.
    if (chunk == 0 && threadIdx.x == 0) {
        if (0 > nY - TB) f |= 1;
        if (nY <= TB) f |= 2;
        if (0 > nX - TB) f |= 4;
        if (nX <= TB) f |= 8;
    }
    return f;
}
// OR of f over the CTA (256 threads), valid in thread 0.
__device__ __forceinline__ int block_or(int f) {
    __shared__ int red;
    if (threadIdx.x == 0) red = 0;
    __syncthreads();
    f = __reduce_or_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && f) atomicOr(&red, f);
    __syncthreads();
    return red;
}

// One word per (tile, chunk): the host ORs a tile's chunks, so nothing needs zeroing.
__global__ void __launch_bounds__(256) k_act_flags(DevArrays A, const int* __restrict__ slots, int qcur, int ts,
                                                    const double* __restrict__ hn_over, int* __restrict__ flags, int per) {
    kg_dep_wait();
    int pos = blockIdx.x / per, chunk = blockIdx.x % per;
    int f = block_or(act_bits(cP, A, slots[pos], qcur, ts, hn_over, chunk));
    if (threadIdx.x == 0) flags[blockIdx.x] = f;
}

// Sequential compensated sums over the active tiles in list order (j outer, i inner).
__global__ void k_volume(DevArrays A, const int* __restrict__ slots, int n, int qcur, int ts, const double* __restrict__ hn_over,
                         const double* __restrict__ rho_over, double* out) {
    const DevParams& P = cP;
    int nX = P.nX, nY = P.nY, SC = nX * nY;
    const double* Q = A.Q[qcur];
    double vol = 0, mass = 0, bed = 0, sol = 0, cv = 0, cm = 0, cb = 0, cs = 0;
    double e2 = P.hThr * P.hThr;
    for (int k = 0; k < n; ++k) {
        int s = slots[k];
        for (int c = 0; c < SC; ++c) {
            double w = Q[pl(s, 4, 0, SC) + c], p = Q[pl(s, 4, 3, SC) + c];
            const double* CT = A.CT[ts];
            double b0 = CT[pl(s, 4, 0, SC) + c], bt = CT[pl(s, 4, 1, SC) + c];
            double gam = gam_of(P.geo, CT[pl(s, 4, 2, SC) + c], CT[pl(s, 4, 3, SC) + c]);
            double Hn, rho;
            if (hn_over) {
                Hn = hn_over[(size_t)s * SC + c];
                rho = rho_over[(size_t)s * SC + c];
            } else {
                Hn = compute_hn(w, b0, bt, gam);
                if (Hn < 0.0) Hn = 0.0;
                double pp = p < 0.0 ? 0.0 : p;
                double psi = mn(2.0 * Hn * pp / (Hn * Hn + mx(Hn * Hn, e2)), P.maxPack);
                rho = density(P, psi);
            }
            double dv = (w - b0 - bt) * gam * gam;
            kahan_add(dv, vol, cv);
            kahan_add(rho * Hn * gam, mass, cm);
            kahan_add(bt, bed, cb);
            kahan_add(p * gam, sol, cs);
        }
    }
    out[0] = vol * P.dx * P.dy;
    out[1] = bed * P.dx * P.dy;
    out[2] = mass * P.dx * P.dy;
    out[3] = sol * P.dx * P.dy;
}

// ---- host launchers ----
cudaError_t launch_cell_topo(const DevArrays& A, const int* d_slots, int n, int ts, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_cell_topo<<<n, 256, 0, st>>>(A, d_slots, ts);
    return cudaGetLastError();
}
static inline int faces_per(int nX, int nY) { return (std::max((nX + 1) * nY, nX * (nY + 1)) + 255) / 256; }
cudaError_t launch_face_bI(const DevArrays& A, const int* d_slots, int n, int ts, int nX, int nY, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int per = faces_per(nX, nY);
    k_face_bI<<<n * per, 256, 0, st>>>(A, d_slots, ts, per);
    return cudaGetLastError();
}
cudaError_t launch_face_topo(const DevArrays& A, const int* d_slots, int n, int ts, int nX, int nY, bool plain, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int per = faces_per(nX, nY);
    if (plain) k_face_topo<true><<<n * per, 256, 0, st>>>(A, d_slots, ts, per);
    else k_face_topo<false><<<n * per, 256, 0, st>>>(A, d_slots, ts, per);
    return cudaGetLastError();
}
cudaError_t launch_ghost_default(const DevArrays& A, int slot, int mode, int ts, cudaStream_t st) {
    k_ghost_bc<<<1, 256, 0, st>>>(A, slot, mode, ts);
    return cudaGetLastError();
}
cudaError_t launch_ghost_dirichlet(const DevArrays& A, int slot, double H, double u, double v, double psi, int ts, cudaStream_t st) {
    k_ghost_dirichlet<<<1, 256, 0, st>>>(A, slot, H, u, v, psi, ts);
    return cudaGetLastError();
}
cudaError_t launch_ghost_edges(const DevArrays& A, int slot, int mask, int qcur, cudaStream_t st) {
    k_ghost_edges<<<1, 256, 0, st>>>(A, slot, mask, qcur);
    return cudaGetLastError();
}
cudaError_t launch_activate(const DevArrays& A, int slot, int qcur, int ts, cudaStream_t st) {
    k_activate<<<1, 256, 0, st>>>(A, slot, qcur, ts);
    return cudaGetLastError();
}
// The state of the listed tiles packed for one read-back: the four conserved planes of
// each tile (w, rhoHnu, rhoHnv, Hnpsi, contiguous per slot) into u4[k][4][SC] and its
// vertex bed change into btv[k][SV], k in list order.
// (In the FP32 form, mom32, the momentum plane holds both momenta as floats; they are
// widened into planes 1 and 2 of the packed state.)
__global__ void __launch_bounds__(256) k_gather_state(DevArrays A, const int* __restrict__ slots, int n, int qcur, int ts,
                                                      int SC, int SV, int mom32, double* __restrict__ u4,
                                                      double* __restrict__ btv) {
    kg_dep_wait();
    const long long per = 4LL * SC + SV, total = per * n;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        int k = (int)(e / per);
        long long r = e - k * per;
        int s = slots[k];
        if (r < 4LL * SC) {
            const double* q = A.Q[qcur] + (size_t)s * 4 * SC;
            double v;
            if (mom32 && r >= SC && r < 3LL * SC) v = (double)reinterpret_cast<const float*>(q + SC)[r - SC];
            else v = q[r];
            u4[(size_t)k * 4 * SC + r] = v;
        } else {
            btv[(size_t)k * SV + (r - 4LL * SC)] = A.BV[ts][((size_t)s * 2 + 1) * SV + (r - 4LL * SC)];
        }
    }
}
cudaError_t launch_gather_state(const DevArrays& A, const int* d_slots, int n, int qcur, int ts, int SC, int SV, bool mom32,
                                double* u4, double* btv, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    long long total = (4LL * SC + SV) * n;
    int grid = (int)std::min<long long>((total + 255) / 256, 152LL * 8);
    KG_TRY_LAUNCH(kg_launch(k_gather_state, grid, 256, 0, st, A, d_slots, n, qcur, ts, SC, SV, mom32 ? 1 : 0, u4, btv));
    return cudaGetLastError();
}
cudaError_t launch_init_maxima(const DevArrays& A, int slot, cudaStream_t st) {
    k_init_maxima<<<1, 256, 0, st>>>(A, slot);
    return cudaGetLastError();
}
cudaError_t launch_act_flags(const DevArrays& A, const int* d_slots, int n, int qcur, int ts, const double* hn_over, int* d_flags,
                             int nX, int nY, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int per = (nX * nY + 255) / 256;
    KG_TRY_LAUNCH(kg_launch(k_act_flags, n * per, 256, 0, st, A, d_slots, qcur, ts, hn_over, d_flags, per));
    return cudaGetLastError();
}
cudaError_t launch_volume(const DevArrays& A, const int* d_slots, int n, int qcur, int ts, const double* hn, const double* rho,
                          double* d_out, cudaStream_t st) {
    k_volume<<<1, 1, 0, st>>>(A, d_slots, n, qcur, ts, hn, rho, d_out);
    return cudaGetLastError();
}

}  // namespace kg
