// kg_engine.cuh -- device data layout shared by the kernels and the host engine.
//
// HBM layout (one "slot" per allocated tile, active or ghost; fields of a slot are
// contiguous planes, x fastest):
//   state buffers  Q[buf][slot][4][nY][nX]    w, rhoHnu, rhoHnv, Hnpsi (buf: 0/1 ping-pong
//                                             solution, 2/3 RK stage results)
//   RHS of stage 1 E0[slot][4][nY][nX], I0[slot][nY][nX]
//   velocities     UV[slot][2][nY][nX]        u, v as the reference leaves them after a step
//   cell topo      CT[slot][4][nY][nX]        b0, bt, dbdx, dbdy at cell centres
//   face topo X    FX[slot][5][nY][nX+1]      b0, bt, dbdx, dbdy, InterpolateB(b0,bt)
//   face topo Y    FY[slot][5][nY+1][nX]
//   vertices       BV[slot][2][nY+1][nX+1]    b0, bt (each tile keeps its own copy of its
//                                             edge vertices, as the reference does)
//   ghost data     G9[slot][9][nY][nX]        static u(1:9) of a ghost tile
//                  GE[slot][12][nE]           its stale w reconstructions at the edges
//   static slopes  B0S[slot][2][nY][nX]       b0 parts of the cell slopes (FP32-form M stages)
//   M step start   M0[slot][3][nY][nX]        FP32 form: Hn, Hn gam, Hnpsi gam of the M input
//                  MF[slot][14][nY][nX]       FP32 form (float): its psi; the stage's Hn, psi,
//                                             rho, bt, dbdx, dbdy and E - D; a second copy
//                                             of the six stage planes (fused M stages)
//                  BVA[slot][nY+1][nX+1]      FP32 form: a second copy of the vertex bt
//   maxima         MX[slot][11][nY][nX]       Hnmax, umax, emax, dmax, psimax (value, time)
//                                             and tfirst (src/Grid.f90:95-102)
// FP32 form only (static per topography set, rebuilt when the set changes):
//   cell factors   TD[slot][3][nY][nX]        b0+bt, 1/gam^2, 1/gam            (FP64)
//                  TF[slot][6][nY][nX]        gam, dbdx, dbdy, gXp1, gXp2, gYp2 (FP32)
//   face factors   TFX[slot][2][nY][nX+1]     gam, (1+dbdy^2)/gam^3            (FP32)
//                  TFY[slot][2][nY+1][nX]     gam, (1+dbdx^2)/gam^3            (FP32)
#pragma once
#include "kg_physics.cuh"

// Redistribution lists of at most this many dependency waves run as one launch per wave
// (every SM takes part); longer ones are walked by a single CTA with barriers between waves.
#ifndef KG_REDIST_WAVE_MAX
#define KG_REDIST_WAVE_MAX 64
#endif

namespace kg {

// Planes of MF (FP32 form).  The fused M stage (k_m_stage32) alternates the six stage
// planes MF_HN..MF_BY with their copies MF_AHN..MF_ABY (plane + MF_ALT).
enum MfPlane { MF_PSI0 = 0, MF_HN, MF_PSI, MF_RHO, MF_BT, MF_BX, MF_BY, MF_EMD,
               MF_AHN, MF_APSI, MF_ARHO, MF_ABT, MF_ABX, MF_ABY, MF_COUNT };
constexpr int MF_ALT = MF_AHN - MF_HN;
enum SlotKind : int8_t { SLOT_FREE = 0, SLOT_ACTIVE = 1, SLOT_GHOST = 2 };
enum Nb { NB_W = 0, NB_E = 1, NB_N = 2, NB_S = 3, NB_SW = 4, NB_SE = 5, NB_NW = 6, NB_NE = 7 };
// Ghost edge records (GE planes): uLimX(iw,1,:), uLimX(iw,nX,:), uLimY(iw,:,1),
// uLimY(iw,:,nY), uPlusX(iw,1,:), uMinusX(iw,2,:), uPlusX(iw,nX,:), uMinusX(iw,nX+1,:),
// uPlusY(iw,:,1), uMinusY(iw,:,2), uPlusY(iw,:,nY), uMinusY(iw,:,nY+1).
enum GEdge { GE_LX1 = 0, GE_LXN, GE_LY1, GE_LYN, GE_PX1, GE_MX2, GE_PXN, GE_MXN1, GE_PY1, GE_MY2, GE_PYN, GE_MYN1, GE_COUNT };

constexpr int MAX_SRC = KG_MAX_SOURCES;
constexpr int MAX_SER = KG_MAX_SERIES;

struct DevSource {
    double x, y, R;
    int n, ncells;
    double time[MAX_SER], flux[MAX_SER], psi[MAX_SER];
};

struct BlockDesc {
    int slot, x0, y0, tile;  // tile: 1-based reference tile ID
};

struct DevArrays {
    int cap;                   // slot capacity
    int nE;                    // max(nX, nY)
    double* Q[4];              // state buffers (the current solution is one of them)
    double* E[2];              // RHS of stage 1 (two sets: step start, and after the M operator)
    double* I[2];
    double* UV;
    double* CT[2];             // topography sets: the step-start bed and the M-updated bed
    double* FX[2];
    double* FY[2];
    double* BV[2];
    double* G9;
    double* GE;
    double* MX;
    double* MS;                // [slot][5][nY][nX] M-operator stage state: w, Hnpsi, Hn, psi, rho
    double* EMD;               // [slot][nY][nX] E - D of the current M stage (zero on ghosts)
    double* B0S;               // [slot][2][nY][nX] the static b0 parts of the cell slopes (FP32-form M stages)
    double* M0;                // [slot][3][nY][nX] FP32 form: the M attempt's step-start Hn (unclamped),
                               // Hn gam and Hnpsi gam (set by m_init, read by the stages and tests)
    float* MF;                 // [slot][14][nY][nX] FP32 form (float): the step-start psi; the M stage's
                               // Hn, psi, rho, bt, dbdx, dbdy as the closures and the vertex source read
                               // them; the stage's E - D (zero on ghosts); the second copy of the six
                               // stage planes that the fused stages alternate with
    double* BVA;               // [slot][nY+1][nX+1] FP32 form: the second copy of the M set's vertex bt
                               // (the fused stages alternate between it and BV[tnew] plane 1)
    double* TD[2];             // FP32 form topography factors (null in the FP64 form)
    float* TF[2];
    float* TFX[2];
    float* TFY[2];
    int* nbr;                  // [cap][8] neighbour slots (-1: none)
    int8_t* kind;              // SlotKind per slot
    int8_t* has_source;        // containsSource per slot
    int* tile_of_slot;         // 1-based tile id
};

// Per-launch control for the fused hydraulic kernels.
enum Mode { MODE_RHS0 = 0, MODE_S1 = 1, MODE_S2 = 2, MODE_S3 = 3 };
struct StepArgs {
    int mode;
    int q_in;        // q0 of the hydraulic step (the reference's intermed0)
    int q_s1;        // S1 writes the stage-2 state here
    int q_s2;        // S2 writes the stage-3 state here (S3 reads it)
    int q_out;       // S3 writes the new solution here
    int e_set;       // E/I set written by RHS0 and read by S1
    int topo;        // topography set of this hydraulic step
    int q_tc, topo_tc;  // the step-start solution (tileContainer) for the maxima
    double dt;       // hydraulic dt of this attempt
    double t_rhs;    // time passed to ConstructHydraulicRHS
    double t_grid;   // grid%t (for the flux-source end-point logic)
    double t_max;    // nextT stamped into the maxima (S3)
    int do_maxima;
    unsigned long long* cfl_min;  // ordered-bits min of the tile CFL terms
    // dt from the device: when dtp is set the pass reads dt there (the advised dt of the
    // step's first RHS evaluation, written by k_dt) and derives t_rhs / t_max from t_grid
    // exactly as the host would (tmode 1: t_rhs = t_grid + dt, 2: t_grid + 0.5 dt;
    // t_max = t_grid + dt).
    const double* dtp;
    int tmode;
    // Stage gate: the pass does nothing when one of these says dt must be refined, so the
    // stages of a step can be queued without waiting for the host's tests in between:
    // gate[g] is a CFL word whose advised dt (with the substep-1 factor 0.9 when
    // gate_s1[g]) falls below dt; gate_flag is a refine flag that is set.
    const unsigned long long* gate[3];
    int gate_s1[3];
    int ngate;
    const int* gate_flag;
    int partial;     // fewer active tiles than tiles: the advised dt is capped by maxdt
};

// Georeferencing of an elevation raster for the vertex-height kernel (kg_dem.cu).
struct RasterGeo {
    long long nx, ny;
    double ox, oy, pw, ph, nodata, ce, cn, dx, dy;
    int nX, nY, nXt, nYt;
};

// Programmatic dependent launch: a kernel launched with kg_launch may be scheduled while
// the previous kernel of the stream drains (hiding the launch gap between the short
// kernels of a step); it calls kg_dep_wait() before touching memory, which returns once
// that kernel has completed and its writes are visible (immediately for a plain launch).
// No kernel signals its dependents early (griddepcontrol.launch_dependents): the next
// kernel's CTAs would then be placed on the SMs that the tail frees first, several per SM,
// instead of spread over all SMs, which costs these FP64-pipe-bound kernels more than the
// launch ramp it saves (measured: step 0.899 -> 0.921 ms).
__device__ __forceinline__ void kg_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
#define KG_TRY_LAUNCH(x)                        \
    do {                                        \
        cudaError_t e_ = (x);                   \
        if (e_ != cudaSuccess) return e_;       \
    } while (0)
template <typename... KArgs, typename... Args>
inline cudaError_t kg_launch(void (*k)(KArgs...), int grid, int block, size_t smem, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

}  // namespace kg
