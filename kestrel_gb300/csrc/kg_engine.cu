// kg_engine.cu -- host engine and C ABI (include/kestrel_gpu.h).
//
// The context owns a pool of tile "slots" in HBM (layout in kg_engine.cuh), the reference's
// tile bookkeeping (active list kept sorted, ghost list in append order, per-tile
// neighbour IDs; src/Grid.f90, src/UpdateTiles.f90) and one CUDA stream.  Per accepted
// step it launches the activation-flag kernel, then the fused hydraulic passes
// (kg_hydro.cu) with the CFL minimum read back after each pass to take the reference's
// accept / refine decisions (src/TimeStepper.f90:151-275).  Tile activation, which in the
// reference mutates the active list while iterating over it, runs on the host from the
// device flags, launching the per-tile set-up kernels (kg_tiles.cu) in the reference's
// order.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "kg_engine.cuh"

namespace kg {
// kg_hydro.cu
size_t hydro_smem_bytes();
cudaError_t set_constants(const DevParams& p, const DevSource* src, int nsrc, cudaStream_t st);
cudaError_t launch_hydro(const DevArrays& A, const BlockDesc* blocks, int nblocks, const StepArgs& S, cudaStream_t st);
// kg_dem.cu
cudaError_t launch_raster_heights(const double* R, const RasterGeo& g, const double* XV, const double* YV, double* out, int* status,
                                  cudaStream_t st);
// kg_tiles.cu
cudaError_t launch_cell_topo(const DevArrays& A, const int* d_slots, int n, int ts, cudaStream_t st);
cudaError_t launch_face_bI(const DevArrays& A, const int* d_slots, int n, int ts, int nX, int nY, cudaStream_t st);
cudaError_t launch_face_topo(const DevArrays& A, const int* d_slots, int n, int ts, int nX, int nY, bool plain, cudaStream_t st);
// kg_hydro32.cu
cudaError_t launch_hydro32(const DevArrays& A, const BlockDesc* blocks, int nblocks, const StepArgs& S, cudaStream_t st);
cudaError_t launch_dt(const unsigned long long* cfl, int partial, double cap, double* dtp, cudaStream_t st);
cudaError_t launch_topo32(const DevArrays& A, const int* d_slots, int n, int ts, int nX, int nY, cudaStream_t st);
cudaError_t launch_ghost_default(const DevArrays& A, int slot, int mode, int ts, cudaStream_t st);
cudaError_t launch_ghost_dirichlet(const DevArrays& A, int slot, double H, double u, double v, double psi, int ts, cudaStream_t st);
cudaError_t launch_ghost_edges(const DevArrays& A, int slot, int mask, int qcur, cudaStream_t st);
cudaError_t launch_activate(const DevArrays& A, int slot, int qcur, int ts, cudaStream_t st);
cudaError_t launch_init_maxima(const DevArrays& A, int slot, cudaStream_t st);
cudaError_t launch_gather_state(const DevArrays& A, const int* d_slots, int n, int qcur, int ts, int SC, int SV, bool mom32,
                                double* u4, double* btv, cudaStream_t st);
cudaError_t launch_act_flags(const DevArrays& A, const int* d_slots, int n, int qcur, int ts, const double* hn_over, int* d_flags,
                             int nX, int nY, cudaStream_t st);
cudaError_t launch_volume(const DevArrays& A, const int* d_slots, int n, int qcur, int ts, const double* hn, const double* rho,
                          double* d_out, cudaStream_t st);
// kg_morpho.cu
cudaError_t launch_m_init(const DevArrays& A, const int* d_slots, int n, int verts, int qa, int tcur, int tnew, int* ctl_flags,
                          bool fp32, cudaStream_t st);
cudaError_t launch_m_emd(const DevArrays& A, const int* d_slots, int n, int cells, int tnew, bool fp32, cudaStream_t st);
int m_stage32_blocks(int nX, int nY);
cudaError_t launch_m_fused32(const DevArrays& A, const int* d_slots, int n, int nX, int nY, int qa, int tcur, int tnew,
                             double dt_m, const double* dtp, int* ctl_flags, unsigned long long* keys, double* ex, int* ncand,
                             int cap, cudaStream_t st);
cudaError_t launch_m_bt(const DevArrays& A, const int* d_slots, int n, int verts, int tcur, int tnew, int stage, double dt,
                        const double* dtp, bool fp32, cudaStream_t st);
cudaError_t launch_m_cells(const DevArrays& A, const int* d_slots, int n, int cells, int qa, int tcur, int tnew, bool fp32,
                           cudaStream_t st);
cudaError_t launch_m_check(const DevArrays& A, const int* d_slots, int n, int cells, int qa, int tcur, int tnew, int* flags,
                           unsigned long long* keys, double* ex, int* ncand, int cap, bool fp32, cudaStream_t st);
cudaError_t launch_m_redist(const DevArrays& A, const int* ls, const int* lc, const int* woff, const int* hwoff, int nwaves,
                            int qa, int tcur, int tnew, int* flags, bool fp32, cudaStream_t st);
cudaError_t launch_m_close(const DevArrays& A, const int* d_slots, int n, int nX, int nY, int qa, int tnew, bool fp32,
                           cudaStream_t st);
}  // namespace kg

using namespace kg;

namespace {

constexpr double HUGE_D = std::numeric_limits<double>::max();
constexpr double PI_D = 3.141592653589793238462643383279502884;

struct KgError : std::runtime_error {
    int code;
    KgError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// A failed CUDA call ends the entry point with its status: KG_ERR_OOM when device memory
// ran out, KG_ERR_CUDA otherwise.
#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            throw KgError(e_ == cudaErrorMemoryAllocation ? KG_ERR_OOM : KG_ERR_CUDA,     \
                          std::string(#call) + ": " + cudaGetErrorString(e_));            \
    } while (0)

struct TileMeta {
    int slot = -1;
    bool on = false, ghost = false, src = false, maxima = false;
    int nb[4] = {0, 0, 0, 0};   // W, E, N, S tile IDs
    int cor[4] = {0, 0, 0, 0};  // SW, SE, NW, NE
};

struct HostSource {
    double x, y, R;
    int n, ncells;
    std::vector<double> time, flux, psi;
};

}  // namespace

struct kg_ctx {
    kg_params p{};
    int prec = KG_PREC_FP64;
    DevParams dp{};
    int nX = 0, nY = 0, nXt = 0, nYt = 0, nTiles = 0, SC = 0, SV = 0, SFX = 0, SFY = 0, nE = 0;
    double xSize = 0, ySize = 0, DeltaT = 0;
    std::vector<TileMeta> tiles;         // index = tile ID - 1
    std::vector<int> active, ghost;      // tile IDs
    std::vector<HostSource> srcs;
    // per-slot host mirrors of the static bed: vertex b0 and face b0 (X, Y)
    std::vector<std::vector<double>> hb0, hfx0, hfy0;
    std::vector<int> slot_tile;
    DevArrays A{};
    int cap = 0, nslots = 0;
    std::vector<BlockDesc> blocks;
    BlockDesc* d_blocks = nullptr;
    int d_blocks_cap = 0;
    int* d_list = nullptr;               // scratch slot list
    int d_list_cap = 0;
    int* d_flags = nullptr;
    int d_flags_cap = 0;
    // Control words the kernels write and the host reads back with one copy per wait:
    // CFL words, the device-chosen dt, the M refine flag and the candidate count.
    struct Ctl {
        unsigned long long cfl[4];
        double dt;
        int mflag, ncand;
    };
    Ctl* d_ctl = nullptr;
    Ctl* h_ctl = nullptr;                // pinned
    unsigned long long* d_cfl = nullptr; // = d_ctl->cfl
    int* d_active = nullptr;             // active slots then ghost slots, list order (device copy)
    int d_active_cap = 0;
    int n_active_dev = -1, n_ghost_dev = 0;
    double* d_vol = nullptr;
    unsigned long long* h_cfl = nullptr; // = h_ctl->cfl
    double* d_dt = nullptr;              // = &d_ctl->dt
    int* h_act = nullptr;                // pinned: edge-band flags read back (per tile chunk)
    int h_act_cap = 0;
    double* d_srcHn = nullptr;           // depth/density the sources set (valid until the first step)
    double* d_srcRho = nullptr;
    bool src_override = false;
    std::vector<double> upload;          // global vertex grid (KG_TOPO_UPLOAD)
    double* d_rb0 = nullptr;             // KG_TOPO_RASTER: every tile's vertex heights (device)
    std::vector<int> raster_status;      // KG_TOPO_RASTER: per tile, 0 ok or the section's failure
    int64_t nx1 = 0, ny1 = 0;
    bool sources_loaded = false;
    int qcur = 0;                        // state buffer holding the solution (0..3)
    int tcur = 0;                        // topography set of the solution (0..1)
    int tdirty[2] = {2, 2};              // FP32 form factor cache of a set: 0 clean, 1 active tiles stale, 2 all stale
    bool fused_m = true;                 // FP32 form: one launch per M stage (k_m_stage32)
    // Edge-band flags of the active tiles computed right after the last accepted hydraulic
    // step on its result (state buffer act_q, topography set act_t), so the next
    // CheckIfNearBoundaries needs no wait of its own; act_gen guards against host writes.
    std::vector<int> act_flags, act_tmp;
    int act_q = -1, act_t = -1;
    int64_t gen = 0, act_gen = -1;
    int* d_tlist = nullptr;              // slot list of the cache rebuild
    int d_tlist_cap = 0;
    double* d_gather = nullptr;          // packed state of the active tiles (kg_get_state)
    size_t d_gather_cap = 0;
    std::vector<int> touched;            // slots whose step-start topography changed in set-up
    int* d_mflags = nullptr;             // = &d_ctl->mflag
    int* d_ncand = nullptr;              // = &d_ctl->ncand
    unsigned long long* d_ckey = nullptr;
    double* d_cex = nullptr;
    int* d_rslot = nullptr;
    int* d_rcell = nullptr;
    int* d_rwave = nullptr;              // wave offsets of the redistribution list
    int cand_cap = 0;
    // Pinned copies of the leading candidates, read back with the control block so that a
    // typical redistribution list needs no second wait; the prefix adapts to the counts seen.
    unsigned long long* h_ckey = nullptr;
    double* h_cex = nullptr;
    int h_cand_cap = 0, cand_pre = 256, cand_pre_used = 0;
    std::vector<std::vector<int>> redist_grid;  // per-tile wave tables of the redistribution scheduler
    double t = 0.0, dt = 1.0e-5, t0 = 0.0;
    int64_t launches = 0, steps = 0, rejected = 0, cell_updates = 0;
    int64_t h2d_bytes = 0, d2h_bytes = 0;  // host<->device traffic of this context
    bool maxima_done = false;              // the running maxima were updated in this step
    int64_t redist_cells = 0, redist_waves = 0, redist_walks = 0;
    // Host wall time (s): whole steps, waiting in stream synchronisations, planning the
    // redistribution walk (read-back of the list excluded).
    double host_step_s = 0.0, host_wait_s = 0.0, host_plan_s = 0.0;
    bool blocks_dirty = true;
    bool timing = false;
    cudaEvent_t ev0[4] = {nullptr, nullptr, nullptr, nullptr}, ev1[4] = {nullptr, nullptr, nullptr, nullptr};
    double kernel_ms = 0.0;
    int64_t timed_passes = 0;
    cudaStream_t st = nullptr;
    std::vector<DevSource> dsrc;         // the source table as uploaded (for re-binding)
    DevSource* d_src = nullptr;          // device copy of the source table (batched passes)
    bool own_stream = true, own_ctl = true;  // false for members of a batch
    std::string err;
};

// Every host<->device copy of a context goes through here and is counted.
cudaError_t kg_cpy(kg_ctx& c, void* dst, const void* src, size_t n, cudaMemcpyKind kind) {
    if (kind == cudaMemcpyHostToDevice) c.h2d_bytes += (int64_t)n;
    else if (kind == cudaMemcpyDeviceToHost) c.d2h_bytes += (int64_t)n;
    return cudaMemcpyAsync(dst, src, n, kind, c.st);
}


namespace {

// The FP32 form keeps the momenta of a slot's state in FP32: its momentum plane (plane 1
// of the slot's four) holds rhoHnu as SC floats followed by rhoHnv as SC floats, and plane
// 2 is unused; the FP64 form keeps four FP64 planes.  These convert one slot's four
// planes between the host's FP64 layout and the context's.
void pack_state(const kg_ctx& c, const double* in, double* out) {
    const size_t SC = (size_t)c.SC;
    if (c.prec != KG_PREC_FP32) {
        std::memmove(out, in, 4 * SC * sizeof(double));
        return;
    }
    std::vector<float> m(2 * SC);
    for (size_t k = 0; k < SC; ++k) {
        m[k] = (float)in[SC + k];
        m[SC + k] = (float)in[2 * SC + k];
    }
    std::memmove(out, in, SC * sizeof(double));
    std::memmove(out + 3 * SC, in + 3 * SC, SC * sizeof(double));
    std::memcpy(out + SC, m.data(), 2 * SC * sizeof(float));
    std::fill(out + 2 * SC, out + 3 * SC, 0.0);
}
void unpack_state(const kg_ctx& c, const double* in, double* out) {
    const size_t SC = (size_t)c.SC;
    if (c.prec != KG_PREC_FP32) {
        std::memmove(out, in, 4 * SC * sizeof(double));
        return;
    }
    std::vector<float> m(2 * SC);
    std::memcpy(m.data(), in + SC, 2 * SC * sizeof(float));
    std::memmove(out, in, SC * sizeof(double));
    std::memmove(out + 3 * SC, in + 3 * SC, SC * sizeof(double));
    for (size_t k = 0; k < SC; ++k) {
        out[SC + k] = (double)m[k];
        out[2 * SC + k] = (double)m[SC + k];
    }
}

// The run settings and source table live in the device's __constant__ bank, shared by
// every context of the process.  The context whose settings are loaded owns it; another
// context re-binds before it launches (after waiting for the owner's stream when the two
// streams differ).  API calls on different contexts are serialised by one lock.
kg_ctx* g_const_owner = nullptr;
std::recursive_mutex g_api_mu;
// Why the calling thread's last kg_create failed (kg_last_error(NULL)); empty after a success.
thread_local std::string g_create_err;

void bind_constants(kg_ctx& c);

// Device bytes of one slot: Q, E/I, CT/FX/FY/BV (two sets), UV, MS, EMD, B0S, G9, GE, MX,
// the source-override Hn and rho planes, nbr/kind/has_source/tile_of_slot, and in the FP32
// form TD/TF/TFX/TFY (two sets), M0/MF and BVA.
size_t slot_bytes(size_t nX, size_t nY, int prec) {
    size_t SC = nX * nY, SFX = (nX + 1) * nY, SFY = nX * (nY + 1), SV = (nX + 1) * (nY + 1), nE = std::max(nX, nY);
    return sizeof(double) * (4 * 4 * SC + 2 * (4 * SC + SC + 4 * SC + 5 * SFX + 5 * SFY + 2 * SV) +
                             2 * SC + 5 * SC + SC + 2 * SC + 9 * SC + GE_COUNT * nE + 11 * SC + 2 * SC) +
           8 * sizeof(int) + 2 + sizeof(int) +
           (prec == KG_PREC_FP32 ? 2 * (3 * sizeof(double) * SC + 6 * sizeof(float) * SC + 2 * sizeof(float) * (SFX + SFY)) +
                                       3 * sizeof(double) * SC + MF_COUNT * sizeof(float) * SC + sizeof(double) * SV
                                 : 0);
}
size_t bytes_per_slot(const kg_ctx& c) { return slot_bytes((size_t)c.nX, (size_t)c.nY, c.prec); }

template <class T>
void grow_array(T*& ptr, size_t old_n, size_t new_n, cudaStream_t st) {
    T* np = nullptr;
    CK(cudaMalloc(&np, new_n * sizeof(T)));
    CK(cudaMemsetAsync(np, 0, new_n * sizeof(T), st));
    if (ptr && old_n) CK(cudaMemcpyAsync(np, ptr, old_n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    if (ptr) {
        CK(cudaStreamSynchronize(st));
        CK(cudaFree(ptr));
    }
    ptr = np;
}

void ensure_cap(kg_ctx& c, int need) {
    if (need <= c.cap) return;
    int nc = std::max(need, std::max(16, c.cap * 2));
    nc = std::min(nc, std::max(need, c.nTiles));
    size_t o = c.cap, n = nc, SC = c.SC;
    for (int b = 0; b < 4; ++b) grow_array(c.A.Q[b], o * 4 * SC, n * 4 * SC, c.st);
    for (int b = 0; b < 2; ++b) {
        grow_array(c.A.E[b], o * 4 * SC, n * 4 * SC, c.st);
        grow_array(c.A.I[b], o * SC, n * SC, c.st);
        grow_array(c.A.CT[b], o * 4 * SC, n * 4 * SC, c.st);
        grow_array(c.A.FX[b], o * 5 * (size_t)c.SFX, n * 5 * (size_t)c.SFX, c.st);
        grow_array(c.A.FY[b], o * 5 * (size_t)c.SFY, n * 5 * (size_t)c.SFY, c.st);
        grow_array(c.A.BV[b], o * 2 * (size_t)c.SV, n * 2 * (size_t)c.SV, c.st);
        if (c.prec == KG_PREC_FP32) {
            grow_array(c.A.TD[b], o * 3 * SC, n * 3 * SC, c.st);
            grow_array(c.A.TF[b], o * 6 * SC, n * 6 * SC, c.st);
            grow_array(c.A.TFX[b], o * 2 * (size_t)c.SFX, n * 2 * (size_t)c.SFX, c.st);
            grow_array(c.A.TFY[b], o * 2 * (size_t)c.SFY, n * 2 * (size_t)c.SFY, c.st);
        }
    }
    if (c.prec == KG_PREC_FP32) {
        grow_array(c.A.M0, o * 3 * SC, n * 3 * SC, c.st);
        grow_array(c.A.MF, o * MF_COUNT * SC, n * MF_COUNT * SC, c.st);
        grow_array(c.A.BVA, o * (size_t)c.SV, n * (size_t)c.SV, c.st);
    }
    grow_array(c.A.UV, o * 2 * SC, n * 2 * SC, c.st);
    grow_array(c.A.MS, o * 5 * SC, n * 5 * SC, c.st);
    grow_array(c.A.EMD, o * SC, n * SC, c.st);
    grow_array(c.A.B0S, o * 2 * SC, n * 2 * SC, c.st);
    grow_array(c.A.G9, o * 9 * SC, n * 9 * SC, c.st);
    grow_array(c.A.GE, o * GE_COUNT * (size_t)c.nE, n * GE_COUNT * (size_t)c.nE, c.st);
    grow_array(c.A.MX, o * 11 * SC, n * 11 * SC, c.st);
    grow_array(c.A.nbr, o * 8, n * 8, c.st);
    grow_array(c.A.kind, o, n, c.st);
    grow_array(c.A.has_source, o, n, c.st);
    grow_array(c.A.tile_of_slot, o, n, c.st);
    grow_array(c.d_srcHn, o * SC, n * SC, c.st);
    grow_array(c.d_srcRho, o * SC, n * SC, c.st);
    c.cap = nc;
    c.A.cap = nc;
    c.hb0.resize(nc);
    c.hfx0.resize(nc);
    c.hfy0.resize(nc);
    c.slot_tile.resize(nc, 0);
}

void ensure_list(kg_ctx& c, size_t n) {
    if ((int)n <= c.d_list_cap) return;
    int nc = std::max<int>((int)n, std::max(64, c.d_list_cap * 2));
    if (c.d_list) CK(cudaFree(c.d_list));
    CK(cudaMalloc(&c.d_list, nc * sizeof(int)));
    c.d_list_cap = nc;
}

void upload_list(kg_ctx& c, const std::vector<int>& slots) {
    ensure_list(c, slots.size());
    if (!slots.empty())
        CK(kg_cpy(c, c.d_list, slots.data(), slots.size() * sizeof(int), cudaMemcpyHostToDevice));
}

double wall() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }
// Edge-band flags are written per (tile, 256-cell chunk).
void ensure_flags(kg_ctx& c, size_t ntiles) {
    size_t need = ntiles * (size_t)((c.SC + 255) / 256);
    if ((int)need <= c.d_flags_cap) return;
    if (c.d_flags) CK(cudaFree(c.d_flags));
    c.d_flags_cap = std::max<int>((int)need, 2 * c.d_flags_cap);
    CK(cudaMalloc(&c.d_flags, (size_t)c.d_flags_cap * sizeof(int)));
}
void sync(kg_ctx& c) {
    double t0 = wall();
    CK(cudaStreamSynchronize(c.st));
    c.host_wait_s += wall() - t0;
}

// ---------------------------------------------------------------- grid navigation
// src/Grid.f90:245-353
int tile_col(const kg_ctx& c, int id) { return (id - 1) % c.nXt + 1; }
int tile_row(const kg_ctx& c, int id) { return (id - 1) / c.nXt + 1; }
int tile_id(const kg_ctx& c, int gi, int gj) { return gi + (gj - 1) * c.nXt; }
bool in_bounds(const kg_ctx& c, int id) { return !(id < 1 || id > c.nTiles); }
bool on_edge(const kg_ctx& c, int id) {
    int i = tile_col(c, id), j = tile_row(c, id);
    bool on = (i == 1 || i == c.nXt);
    return on || (c.nYt > 1 && (j == 1 || j == c.nYt));
}
TileMeta& T(kg_ctx& c, int id) { return c.tiles[(size_t)id - 1]; }
double cell_x(const kg_ctx& c, int gi, int ii) { return -0.5 * c.xSize + c.dp.dx * ((gi - 1.0) * c.nX + (ii - 0.5)); }
double cell_y(const kg_ctx& c, int gj, int jj) { return -0.5 * c.ySize + c.dp.dy * ((gj - 1.0) * c.nY + (jj - 0.5)); }

// SetTileBoundaries / SetPeriodicBoundaryConds, src/UpdateTiles.f90:487-566.
void set_tile_boundaries(kg_ctx& c, int k) {
    TileMeta& m = T(c, k);
    int N = k + c.nXt, S = k - c.nXt;
    m.nb[0] = k - 1; m.nb[1] = k + 1; m.nb[2] = N; m.nb[3] = S;
    m.cor[0] = S - 1; m.cor[1] = S + 1; m.cor[2] = N - 1; m.cor[3] = N + 1;
    if (c.p.bcs == KG_BC_PERIODIC) {
        int gi = tile_col(c, k), gj = tile_row(c, k);
        if (gi == 1) {
            m.nb[0] = tile_id(c, c.nXt, gj);
            if (gj > 1 && gj < c.nYt) { m.cor[0] = tile_id(c, c.nXt, gj - 1); m.cor[2] = tile_id(c, c.nXt, gj + 1); }
            else if (gj == 1) { m.cor[0] = tile_id(c, c.nXt, c.nYt); m.cor[2] = tile_id(c, c.nXt, gj + 1); }
            else if (gj == c.nYt) { m.cor[0] = tile_id(c, c.nXt, gj - 1); m.cor[2] = tile_id(c, c.nXt, 1); }
        }
        if (gi == c.nXt) {
            m.nb[1] = tile_id(c, 1, gj);
            if (gj > 1 && gj < c.nYt) { m.cor[1] = tile_id(c, 1, gj - 1); m.cor[3] = tile_id(c, 1, gj + 1); }
            else if (gj == 1) { m.cor[1] = tile_id(c, 1, c.nYt); m.cor[3] = tile_id(c, 1, gj + 1); }
            else if (gj == c.nYt) { m.cor[1] = tile_id(c, 1, gj - 1); m.cor[3] = tile_id(c, 1, 1); }
        }
        if (gj == 1) m.nb[3] = tile_id(c, gi, c.nYt);
        if (gj == c.nYt) m.nb[2] = tile_id(c, gi, 1);
    }
}

// Neighbour slot table entries of one tile (refreshed whenever a neighbour gets a slot).
void push_nbr(kg_ctx& c, int id) {
    TileMeta& m = T(c, id);
    if (m.slot < 0) return;
    int v[8];
    const int order[8] = {m.nb[0], m.nb[1], m.nb[2], m.nb[3], m.cor[0], m.cor[1], m.cor[2], m.cor[3]};
    for (int q = 0; q < 8; ++q) v[q] = in_bounds(c, order[q]) ? T(c, order[q]).slot : -1;
    CK(kg_cpy(c, c.A.nbr + (size_t)m.slot * 8, v, sizeof(v), cudaMemcpyHostToDevice));
    sync(c);
}
void refresh_nbrs_around(kg_ctx& c, int id) {
    push_nbr(c, id);
    TileMeta& m = T(c, id);
    for (int q = 0; q < 4; ++q)
        if (in_bounds(c, m.nb[q])) push_nbr(c, m.nb[q]);
    for (int q = 0; q < 4; ++q)
        if (in_bounds(c, m.cor[q])) push_nbr(c, m.cor[q]);
    // tiles that list this tile as a neighbour's neighbour (corner relations) are covered
    // by refreshing all slots lazily before each step.
}
void refresh_all_nbrs(kg_ctx& c) {
    std::vector<int> v((size_t)c.nslots * 8, -1);
    for (int s = 0; s < c.nslots; ++s) {
        int id = c.slot_tile[s];
        if (id <= 0) continue;
        TileMeta& m = T(c, id);
        const int order[8] = {m.nb[0], m.nb[1], m.nb[2], m.nb[3], m.cor[0], m.cor[1], m.cor[2], m.cor[3]};
        for (int q = 0; q < 8; ++q) v[(size_t)s * 8 + q] = in_bounds(c, order[q]) ? T(c, order[q]).slot : -1;
    }
    if (!v.empty()) CK(kg_cpy(c, c.A.nbr, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice));
    sync(c);
}

int assign_slot(kg_ctx& c, int id) {
    TileMeta& m = T(c, id);
    if (m.slot >= 0) return m.slot;
    ensure_cap(c, c.nslots + 1);
    int s = c.nslots++;
    m.slot = s;
    c.slot_tile[s] = id;
    int8_t z = SLOT_FREE;
    CK(kg_cpy(c, c.A.kind + s, &z, 1, cudaMemcpyHostToDevice));
    CK(kg_cpy(c, c.A.tile_of_slot + s, &id, sizeof(int), cudaMemcpyHostToDevice));
    sync(c);
    return s;
}
void set_kind(kg_ctx& c, int id, int8_t k) {
    CK(kg_cpy(c, c.A.kind + T(c, id).slot, &k, 1, cudaMemcpyHostToDevice));
    sync(c);
}

// ---------------------------------------------------------------- bed set-up
// GetHeights (src/dem.f90:360-391) with the analytic surfaces of src/TopogFuncs.f90 or the
// uploaded vertex grid, evaluated at the vertex coordinates AllocateTopographicData builds
// (src/UpdateTiles.f90:271-337).
// The remaining analytic surfaces of src/TopogFuncs.f90 at one vertex (X, Y): x2slopes
// (:101-135), usgs (:145-183), flume (:197-242), channel_powerlaw (:255-276),
// channel_trapezium (:288-308), xbislope (:315-337), xtrislope (:346-388).
inline double more_topo(int kind, const double* P, double X, double Y) {
    const double pi = PI_D;
    switch (kind) {
        case KG_TOPO_X2SLOPES: {
            double alpha = P[0], beta = P[1], R = P[2];
            double xc0 = (std::sqrt(1.0 + alpha * alpha) - std::sqrt(1.0 + beta * beta)) * R / (alpha - beta);
            double zc0 = (alpha * std::sqrt(1.0 + beta * beta) - beta * std::sqrt(1.0 + alpha * alpha)) * R / (alpha - beta);
            double x1 = xc0 - alpha * R / std::sqrt(1.0 + alpha * alpha);
            double x2 = xc0 - beta * R / std::sqrt(1.0 + beta * beta);
            if (X < x1) return -alpha * X;
            if (X > x2) return -beta * X;
            return zc0 - std::sqrt(R * R - (X - xc0) * (X - xc0));
        }
        case KG_TOPO_USGS:
        case KG_TOPO_FLUME: {
            double th0 = 31.0, th1 = 2.4, xwall = 8.5, ww = 2.0, wallH = P[0], sigma = P[1];
            if (kind == KG_TOPO_FLUME) { th0 = P[0]; th1 = P[1]; xwall = P[2]; ww = P[3]; wallH = P[4]; sigma = P[5]; }
            double alpha = 8.5 / (std::asinh(-std::tan(4.0 * pi / 180.0)) - std::asinh(-std::tan(th0 * pi / 180.0)));
            double xc0 = -alpha * std::asinh(-std::tan(th0 * pi / 180.0));
            double zc0 = -alpha * std::cosh((-xc0) / alpha);
            double x1 = xc0 + alpha * std::asinh(-std::tan(th1 * pi / 180.0));
            double b;
            if (X < 0.0) b = -std::tan(th0 * pi / 180.0) * X;
            else if (X > x1) b = zc0 + alpha * std::cosh((x1 - xc0) / alpha) - std::tan(th1 * pi / 180.0) * (X - x1);
            else b = zc0 + alpha * std::cosh((X - xc0) / alpha);
            if (X < xwall) {
                if (kind == KG_TOPO_USGS)
                    b = b + 0.5 * wallH * (std::tanh(sigma * (Y - 1.0)) - std::tanh(sigma * (Y - 2.0)) + std::tanh(sigma * (Y + 2.0)) -
                                           std::tanh(sigma * (Y + 1.0)));
                else
                    b = b + 0.5 * wallH * (std::tanh(sigma * (Y - 0.5 * ww)) - std::tanh(sigma * (Y - 1.5 * ww)) +
                                           std::tanh(sigma * (Y + 1.5 * ww)) - std::tanh(sigma * (Y + 0.5 * ww)));
            }
            return b;
        }
        case KG_TOPO_CHANNEL_POWERLAW: {
            double slope = P[0], W = P[1], alpha = P[2];
            double costheta = std::cos(std::atan(slope));
            return slope * X + costheta * std::pow(std::fabs(Y) / W, alpha);
        }
        case KG_TOPO_CHANNEL_TRAPEZIUM: {
            double slope = P[0], W = P[1], Sb = P[2];
            double costheta = std::cos(std::atan(slope));
            return slope * X + costheta * std::max(0.0, Sb * (std::fabs(Y) - 0.5 * W));
        }
        case KG_TOPO_XBISLOPE: {
            double phi1 = P[0] * pi / 180.0, phi2 = P[1] * pi / 180.0, lam = P[2];
            double a1 = std::tan(phi1), a2 = std::tan(phi2);
            return -0.5 * (a1 + a2) * X + 0.5 * (a1 - a2) * lam * std::log(std::cosh(X / lam));
        }
        case KG_TOPO_XTRISLOPE: {
            double phi1 = P[0] * pi / 180.0, phi2 = P[1] * pi / 180.0, phi3 = P[2] * pi / 180.0;
            double lam = P[3], x1 = P[4], x2 = P[5];
            double s1 = std::tan(phi1), s2 = std::tan(phi2), s3 = std::tan(phi3);
            double c2 = (x1 - 0.5 * lam) * 0.5 * (s1 - s2);
            double c3 = (x1 + 0.5 * lam) * 0.5 * (s1 - s2) + c2;
            double c4 = (x2 - 0.5 * lam) * 0.5 * (s2 - s3) + c3;
            double c5 = (x2 + 0.5 * lam) * 0.5 * (s2 - s3) + c4;
            if (X < x1 - 0.5 * lam) return s1 * X;
            if (X < x1 + 0.5 * lam) {
                double A = 0.5 * (s2 - s1) * lam / pi;
                return A * std::sin((X - x1) * pi / lam - 0.5 * pi) + 0.5 * (s1 + s2) * X + c2;
            }
            if (X < x2 - 0.5 * lam) return s2 * X + c3;
            if (X < x2 + 0.5 * lam) {
                double A = 0.5 * (s3 - s2) * lam / pi;
                return A * std::sin((X - x2) * pi / lam - 0.5 * pi) + 0.5 * (s2 + s3) * X + c4;
            }
            return s3 * X + c5;
        }
    }
    return 0.0;
}
double topo_value(const kg_ctx& c, int id, int a, int b, double X, double Y) {
    const double* P = c.p.topog_params;
    switch (c.p.topog) {
        case KG_TOPO_FLAT: return 0.0;
        case KG_TOPO_XSLOPE: return P[0] * X;
        case KG_TOPO_YSLOPE: return P[0] * Y;
        case KG_TOPO_XYSLOPE: return P[0] * X + P[1] * Y;
        case KG_TOPO_XSINSLOPE: {
            double Lx = c.p.Xtilesize * c.nXt;
            double k = 2.0 * PI_D / Lx;
            return P[0] * std::sin(X * k);
        }
        case KG_TOPO_XYSINSLOPE: {
            double Lx = c.p.Xtilesize * c.nXt, Ly = c.p.Ytilesize * c.nYt;
            double kx = 2.0 * PI_D / Lx, ky = 2.0 * PI_D / Ly;
            return P[0] * std::sin(X * kx) * std::sin(Y * ky);
        }
        case KG_TOPO_XHUMP: return ((X > -P[1]) && (X < P[1])) ? 0.5 * P[0] * (1.0 + std::cos(PI_D * X / P[1])) : 0.0;
        case KG_TOPO_XTANH: return P[1] * (1.0 + std::tanh((X - P[0]) / P[2]));
        case KG_TOPO_XPARAB: return P[0] * X * X;
        case KG_TOPO_XYPARAB: return P[0] * X * X + P[1] * Y * Y;
        case KG_TOPO_X2SLOPES:
        case KG_TOPO_USGS:
        case KG_TOPO_FLUME:
        case KG_TOPO_CHANNEL_POWERLAW:
        case KG_TOPO_CHANNEL_TRAPEZIUM:
        case KG_TOPO_XBISLOPE:
        case KG_TOPO_XTRISLOPE: return more_topo(c.p.topog, P, X, Y);
        default: {
            int gi = tile_col(c, id), gj = tile_row(c, id);
            int64_t vx = (int64_t)(gi - 1) * c.nX + a, vy = (int64_t)(gj - 1) * c.nY + b;
            return c.upload[(size_t)(vx + c.nx1 * vy)];
        }
    }
}
// Vertex coordinates of tile column gi / row gj (x_vertex, y_vertex of
// src/UpdateTiles.f90:308-325).
void vertex_x(const kg_ctx& c, int gi, double* xv) {
    for (int ii = 1; ii <= c.nX; ++ii) xv[ii - 1] = cell_x(c, gi, ii) - 0.5 * c.dp.dx;
    xv[c.nX] = cell_x(c, gi, c.nX) + 0.5 * c.dp.dx;
}
void vertex_y(const kg_ctx& c, int gj, double* yv) {
    for (int jj = 1; jj <= c.nY; ++jj) yv[jj - 1] = cell_y(c, gj, jj) - 0.5 * c.dp.dy;
    yv[c.nY] = cell_y(c, gj, c.nY) + 0.5 * c.dp.dy;
}
void get_heights(kg_ctx& c, int id) {
    int s = T(c, id).slot, nX = c.nX, nY = c.nY, gi = tile_col(c, id), gj = tile_row(c, id);
    std::vector<double> xv(nX + 1), yv(nY + 1);
    vertex_x(c, gi, xv.data());
    vertex_y(c, gj, yv.data());
    std::vector<double>& b0 = c.hb0[s];
    b0.assign((size_t)c.SV, 0.0);
    if (c.p.topog == KG_TOPO_RASTER) {
        // The raster section read fails as in GeoTiffArraySectionRead (src/GeoTiffRead.f90:213-214).
        int st = c.raster_status[(size_t)id - 1];
        if (st == 1) throw KgError(KG_ERR_PARAM, "Could not read raster file: the section of tile " + std::to_string(id) + " leaves the raster");
        if (st == 2) throw KgError(KG_ERR_PARAM, "No-data value found in raster file (section of tile " + std::to_string(id) + ")");
        if (st != 0) throw KgError(KG_ERR_PARAM, "raster section of tile " + std::to_string(id) + " too small for its bicubic samples");
        CK(kg_cpy(c, b0.data(), c.d_rb0 + (size_t)(id - 1) * c.SV, (size_t)c.SV * sizeof(double), cudaMemcpyDeviceToHost));
        sync(c);
    } else {
        for (int b = 0; b <= nY; ++b)
            for (int a = 0; a <= nX; ++a) b0[(size_t)b * (nX + 1) + a] = topo_value(c, id, a, b, xv[a], yv[b]);
    }
    c.hfx0[s].assign((size_t)c.SFX, 0.0);
    c.hfy0[s].assign((size_t)c.SFY, 0.0);
    for (int j = 0; j < nY; ++j)
        for (int a = 0; a <= nX; ++a)
            c.hfx0[s][(size_t)j * (nX + 1) + a] = 0.5 * (b0[(size_t)j * (nX + 1) + a] + b0[(size_t)(j + 1) * (nX + 1) + a]);
    for (int a = 0; a <= nY; ++a)
        for (int i = 0; i < nX; ++i)
            c.hfy0[s][(size_t)a * nX + i] = 0.5 * (b0[(size_t)a * (nX + 1) + i] + b0[(size_t)a * (nX + 1) + i + 1]);
}
void push_bed(kg_ctx& c, int s) {
    // b0 and the face b0 are static: both topography sets hold them.
    for (int b = 0; b < 2; ++b) {
        CK(kg_cpy(c, c.A.BV[b] + (size_t)s * 2 * c.SV, c.hb0[s].data(), (size_t)c.SV * sizeof(double), cudaMemcpyHostToDevice));
        CK(kg_cpy(c, c.A.FX[b] + (size_t)s * 5 * c.SFX, c.hfx0[s].data(), (size_t)c.SFX * sizeof(double), cudaMemcpyHostToDevice));
        CK(kg_cpy(c, c.A.FY[b] + (size_t)s * 5 * c.SFY, c.hfy0[s].data(), (size_t)c.SFY * sizeof(double), cudaMemcpyHostToDevice));
    }
}
void touch(kg_ctx& c, int s) {
    c.tdirty[0] = c.tdirty[1] = 2;
    if (std::find(c.touched.begin(), c.touched.end(), s) == c.touched.end()) c.touched.push_back(s);
}
// The second topography set of a slot is scratch for active tiles during a step and a
// copy of the first for ghost tiles; after set-up work the touched slots are mirrored.
void mirror_touched(kg_ctx& c) {
    int o = 1 - c.tcur;
    for (int s : c.touched) {
        CK(kg_cpy(c, c.A.CT[o] + (size_t)s * 4 * c.SC, c.A.CT[c.tcur] + (size_t)s * 4 * c.SC, (size_t)4 * c.SC * sizeof(double), cudaMemcpyDeviceToDevice));
        CK(kg_cpy(c, c.A.FX[o] + (size_t)s * 5 * c.SFX, c.A.FX[c.tcur] + (size_t)s * 5 * c.SFX, (size_t)5 * c.SFX * sizeof(double), cudaMemcpyDeviceToDevice));
        CK(kg_cpy(c, c.A.FY[o] + (size_t)s * 5 * c.SFY, c.A.FY[c.tcur] + (size_t)s * 5 * c.SFY, (size_t)5 * c.SFY * sizeof(double), cudaMemcpyDeviceToDevice));
        CK(kg_cpy(c, c.A.BV[o] + (size_t)s * 2 * c.SV, c.A.BV[c.tcur] + (size_t)s * 2 * c.SV, (size_t)2 * c.SV * sizeof(double), cudaMemcpyDeviceToDevice));
    }
    c.touched.clear();
    sync(c);
}
// ComputeCellCentredTopographicData for a tile after its vertex b0 changed; InterpolateB
// is recomputed with it since the reference evaluates that from the vertices on use.
void cell_topo(kg_ctx& c, int id) {
    int s = T(c, id).slot;
    push_bed(c, s);
    std::vector<int> one{s};
    upload_list(c, one);
    CK(launch_cell_topo(c.A, c.d_list, 1, c.tcur, c.st));
    CK(launch_face_bI(c.A, c.d_list, 1, c.tcur, c.nX, c.nY, c.st));
    c.launches += 2;
    touch(c, s);
    sync(c);
}
bool in_list(const std::vector<int>& v, int x) { return std::find(v.begin(), v.end(), x) != v.end(); }
bool is_active_ghost(kg_ctx& c, int id) { return in_list(c.ghost, id) && T(c, id).ghost; }

// EqualiseTopographicBoundaryData, src/MorphodynamicRHS.f90:588-687 (vertex and face b0).
void equalise(kg_ctx& c, int id) {
    c.tdirty[0] = c.tdirty[1] = 2;
    int nX = c.nX, nY = c.nY, V = nX + 1;
    auto ok = [&](int t) { return in_bounds(c, t) && (in_list(c.active, t) || is_active_ghost(c, t)); };
    auto B0 = [&](int t) -> std::vector<double>& { return c.hb0[T(c, t).slot]; };
    auto FX0 = [&](int t) -> std::vector<double>& { return c.hfx0[T(c, t).slot]; };
    auto FY0 = [&](int t) -> std::vector<double>& { return c.hfy0[T(c, t).slot]; };
    bool sw_up = false, ne_up = false;
    int tW = T(c, id).nb[0];
    if (ok(tW)) {
        for (int j = 0; j < nY; ++j) {
            B0(tW)[(size_t)j * V + nX] = B0(id)[(size_t)j * V + 0];
            FX0(tW)[(size_t)j * V + nX] = FX0(id)[(size_t)j * V + 0];
        }
        cell_topo(c, tW);
        int tSW = T(c, tW).nb[3];
        if (ok(tSW)) {
            B0(tSW)[(size_t)nY * V + nX] = B0(id)[0];
            sw_up = true;
            cell_topo(c, tSW);
        }
    }
    int tE = T(c, id).nb[1];
    if (ok(tE)) {
        for (int j = 0; j < nY; ++j) {
            B0(id)[(size_t)j * V + nX] = B0(tE)[(size_t)j * V + 0];
            FX0(id)[(size_t)j * V + nX] = FX0(tE)[(size_t)j * V + 0];
        }
        int tNE = T(c, tE).nb[2];
        if (ok(tNE)) {
            B0(id)[(size_t)nY * V + nX] = B0(tNE)[0];
            ne_up = true;
        }
        cell_topo(c, id);
    }
    int tN = T(c, id).nb[2];
    if (ok(tN)) {
        for (int i = 0; i < nX; ++i) {
            B0(id)[(size_t)nY * V + i] = B0(tN)[i];
            FY0(id)[(size_t)nY * nX + i] = FY0(tN)[i];
        }
        if (!ne_up) {
            int tNE = T(c, tN).nb[1];
            if (ok(tNE)) B0(id)[(size_t)nY * V + nX] = B0(tNE)[0];
        }
        cell_topo(c, id);
    }
    int tS = T(c, id).nb[3];
    if (ok(tS)) {
        for (int i = 0; i < nX; ++i) {
            B0(tS)[(size_t)nY * V + i] = B0(id)[i];
            FY0(tS)[(size_t)nY * nX + i] = FY0(id)[i];
        }
        cell_topo(c, tS);
        if (!sw_up) {
            int tSW = T(c, tS).nb[0];
            if (ok(tSW)) {
                B0(tSW)[(size_t)nY * V + nX] = B0(id)[0];
                cell_topo(c, tSW);
            }
        }
    }
}

// ReconstructwAtEdges (src/UpdateTiles.f90:669-750) for a ghost tile: each edge whose
// neighbour is on gets its limited w slope and face reconstructions from current data.
void ghost_edges(kg_ctx& c, int gid) {
    TileMeta& m = T(c, gid);
    int mask = 0;
    const int dirs[4] = {m.nb[0], m.nb[1], m.nb[3], m.nb[2]};  // W, E, S, N
    for (int q = 0; q < 4; ++q)
        if (in_bounds(c, dirs[q]) && T(c, dirs[q]).on) mask |= (1 << q);
    if (!mask) return;
    CK(launch_ghost_edges(c.A, m.slot, mask, c.qcur, c.st));
    c.launches++;
    sync(c);
}

// AllocateU + AllocateTopographicData + SetTileBoundaries + GetHeights + the cell data.
void init_tile_geometry(kg_ctx& c, int id) {
    assign_slot(c, id);
    set_tile_boundaries(c, id);
    refresh_nbrs_around(c, id);
    get_heights(c, id);
    cell_topo(c, id);
}

void add_tile(kg_ctx& c, int k);

// AddGhostTiles, src/UpdateTiles.f90:389-481.
void add_ghost_tiles(kg_ctx& c, int k) {
    std::vector<int> fresh;
    for (int i = 1; i <= 8; ++i) {
        int tile;
        if (i > 4) {
            if (c.p.bcs == KG_BC_PERIODIC) break;
            tile = T(c, k).cor[i - 5];
        } else {
            tile = T(c, k).nb[i - 1];
        }
        if (!in_bounds(c, tile)) throw KgError(KG_ERR_HALT_EDGE, "a ghost tile would lie outside the domain");
        bool already = in_list(c.ghost, tile);
        if (already) ghost_edges(c, tile);
        else if (!T(c, tile).on && !in_list(fresh, tile)) fresh.push_back(tile);
    }
    if (fresh.empty()) return;
    for (int t : fresh) c.ghost.push_back(t);
    for (int t : fresh) {
        init_tile_geometry(c, t);
        int s = T(c, t).slot;
        if (on_edge(c, t)) {
            if (c.p.bcs == KG_BC_DIRICHLET)
                CK(launch_ghost_dirichlet(c.A, s, c.p.bcsHnval, c.p.bcsuval, c.p.bcsvval, c.p.bcspsival, c.tcur, c.st));
            else
                CK(launch_ghost_default(c.A, s, c.p.bcs == KG_BC_PERIODIC ? 2 : 0, c.tcur, c.st));
        } else {
            CK(launch_ghost_default(c.A, s, 0, c.tcur, c.st));
        }
        c.launches++;
        sync(c);
        ghost_edges(c, t);
        T(c, t).ghost = true;
        set_kind(c, t, SLOT_GHOST);
    }
    for (int t : fresh) equalise(c, t);
}

// AddTile / AddToActiveTiles / AllocateTile / ActivateTile, src/UpdateTiles.f90:56-384.
void add_tile(kg_ctx& c, int k) {
    if (!in_bounds(c, k) || (on_edge(c, k) && c.p.bcs != KG_BC_PERIODIC)) {
        if (c.p.bcs == KG_BC_HALT)
            throw KgError(KG_ERR_HALT_EDGE, "tried to add a tile outside the domain (increase the domain size)");
        return;
    }
    // AddToActiveTiles (sorted insert; a ghost tile leaves the ghost list).
    if (!in_list(c.active, k)) {
        auto pos = std::upper_bound(c.active.begin(), c.active.end(), k);
        c.active.insert(pos, k);
        auto it = std::find(c.ghost.begin(), c.ghost.end(), k);
        if (it != c.ghost.end()) {
            c.ghost.erase(it);
            T(c, k).ghost = false;
        }
    }
    // AllocateTile
    TileMeta& m = T(c, k);
    m.on = true;
    init_tile_geometry(c, k);
    if (!T(c, k).maxima) {
        CK(launch_init_maxima(c.A, T(c, k).slot, c.st));
        c.launches++;
        T(c, k).maxima = true;
    }
    equalise(c, k);
    T(c, k).src = false;
    int8_t zero = 0;
    CK(kg_cpy(c, c.A.has_source + T(c, k).slot, &zero, 1, cudaMemcpyHostToDevice));
    // ActivateTile
    T(c, k).ghost = false;
    set_kind(c, k, SLOT_ACTIVE);
    CK(launch_activate(c.A, T(c, k).slot, c.qcur, c.tcur, c.st));
    touch(c, T(c, k).slot);
    c.launches++;
    sync(c);
    add_ghost_tiles(c, k);
    std::vector<int> one{T(c, k).slot};
    upload_list(c, one);
    CK(launch_face_topo(c.A, c.d_list, 1, c.tcur, c.nX, c.nY, false, c.st));
    c.launches++;
    sync(c);
    c.blocks_dirty = true;
    c.tdirty[0] = c.tdirty[1] = 2;
}

void rebuild_blocks(kg_ctx& c) {
    if (!c.blocks_dirty) return;
    refresh_all_nbrs(c);
    // Device copy of the slot lists: active tiles in list order, then the ghost tiles.
    std::vector<int> all;
    for (int id : c.active) all.push_back(T(c, id).slot);
    for (int id : c.ghost) all.push_back(T(c, id).slot);
    if ((int)all.size() > c.d_active_cap) {
        if (c.d_active) CK(cudaFree(c.d_active));
        c.d_active_cap = std::max<int>((int)all.size(), 2 * c.d_active_cap);
        CK(cudaMalloc(&c.d_active, (size_t)c.d_active_cap * sizeof(int)));
    }
    if (!all.empty()) CK(kg_cpy(c, c.d_active, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice));
    c.n_active_dev = (int)c.active.size();
    c.n_ghost_dev = (int)c.ghost.size();
    c.blocks.clear();
    const int BSZ = 16;
    for (int id : c.active) {
        int s = T(c, id).slot;
        for (int y0 = 0; y0 < c.nY; y0 += BSZ)
            for (int x0 = 0; x0 < c.nX; x0 += BSZ) c.blocks.push_back(BlockDesc{s, x0, y0, id});
    }
    if ((int)c.blocks.size() > c.d_blocks_cap) {
        if (c.d_blocks) CK(cudaFree(c.d_blocks));
        c.d_blocks_cap = std::max<int>((int)c.blocks.size(), 2 * c.d_blocks_cap);
        CK(cudaMalloc(&c.d_blocks, (size_t)c.d_blocks_cap * sizeof(BlockDesc)));
    }
    if (!c.blocks.empty())
        CK(kg_cpy(c, c.d_blocks, c.blocks.data(), c.blocks.size() * sizeof(BlockDesc), cudaMemcpyHostToDevice));
    sync(c);
    c.blocks_dirty = false;
}

// CheckIfNearBoundaries, src/TimeStepper.f90:924-1150: device edge-band flags for the
// tiles active at the start of the check, then the reference's four sweeps with the list
// growing (and shifting) under the loop; tiles added during the sweeps are dry.
void check_near_boundaries(kg_ctx& c) {
    if (c.active.empty()) return;
    std::vector<int> slots;
    for (int id : c.active) slots.push_back(T(c, id).slot);
    std::vector<int> fl;
    if (!c.src_override && c.act_q == c.qcur && c.act_t == c.tcur && c.act_gen == c.gen && c.act_flags.size() == slots.size()) {
        fl = c.act_flags;
    } else {
        upload_list(c, slots);
        ensure_flags(c, slots.size());
        CK(launch_act_flags(c.A, c.d_list, (int)slots.size(), c.qcur, c.tcur, c.src_override ? c.d_srcHn : nullptr, c.d_flags, c.nX, c.nY, c.st));
        c.launches++;
        int per = (c.SC + 255) / 256;
        std::vector<int> chunks(slots.size() * per);
        CK(kg_cpy(c, chunks.data(), c.d_flags, chunks.size() * sizeof(int), cudaMemcpyDeviceToHost));
        sync(c);
        fl.assign(slots.size(), 0);
        for (size_t q = 0; q < slots.size(); ++q)
            for (int k = 0; k < per; ++k) fl[q] |= chunks[q * per + k];
    }
    c.act_q = -1;
    std::vector<int> flag_of((size_t)c.nTiles + 1, -1);
    for (size_t q = 0; q < slots.size(); ++q) flag_of[(size_t)c.active[q]] = fl[q];
    int TB = c.p.TileBuffer;
    int dry_flags = (0 > c.nY - TB ? 1 : 0) | (c.nY <= TB ? 2 : 0) | (0 > c.nX - TB ? 4 : 0) | (c.nX <= TB ? 8 : 0);
    // Sweep order N, S, E, W with neighbour index 2, 3, 1, 0.
    const int bit[4] = {1, 2, 4, 8}, nbi[4] = {2, 3, 1, 0};
    for (int d = 0; d < 4; ++d) {
        int size0 = (int)c.active.size();
        for (int tt = 0; tt < size0; ++tt) {
            int ttk = c.active[(size_t)tt];
            int nbt = T(c, ttk).nb[nbi[d]];
            if (nbt > 0 && in_bounds(c, nbt) && !T(c, nbt).on) {
                int f = flag_of[(size_t)ttk];
                if (f < 0) f = dry_flags;
                if (f & bit[d]) add_tile(c, nbt);
            }
        }
    }
    if (!c.touched.empty()) mirror_touched(c);
}

// ComputeAdvisedTimeStep, src/HydraulicRHS.f90:141-174.
double advised(kg_ctx& c, unsigned long long bits, int substep) {
    double umin;
    std::memcpy(&umin, &bits, sizeof(double));
    if ((int)c.active.size() < c.nTiles) umin = mn(umin, c.p.maxdt);
    double m = mn(c.p.cfl * umin, c.dp.diffusiveTimeScale);
    m = mn(m, c.p.maxdt);
    if (substep == 1) return 0.9 * m;
    return m;
}

// Before the constant bank is rewritten for context c, the kernels the previous owner
// queued on another stream (which read the bank) must have finished.
void wait_const_owner(kg_ctx& c) {
    if (g_const_owner && g_const_owner != &c && g_const_owner->st != c.st) CK(cudaStreamSynchronize(g_const_owner->st));
}

void bind_constants(kg_ctx& c) {
    if (g_const_owner == &c) return;
    wait_const_owner(c);
    CK(set_constants(c.dp, c.dsrc.empty() ? nullptr : c.dsrc.data(), (int)c.dsrc.size(), c.st));
    g_const_owner = &c;
}

// FP32 form: rebuild the factor cache of topography set ts for every allocated tile.
void refresh_topo32(kg_ctx& c, int ts) {
    if (c.n_active_dev == (int)c.active.size() && c.n_ghost_dev == (int)c.ghost.size() && !c.blocks_dirty) {
        int n = c.n_active_dev + (c.tdirty[ts] > 1 ? c.n_ghost_dev : 0);
        if (n > 0) {
            CK(launch_topo32(c.A, c.d_active, n, ts, c.nX, c.nY, c.st));
            c.launches++;
        }
        c.tdirty[ts] = 0;
        return;
    }
    std::vector<int> slots;
    for (int id : c.active) slots.push_back(T(c, id).slot);
    if (c.tdirty[ts] > 1)
        for (int id : c.ghost) slots.push_back(T(c, id).slot);
    if ((int)slots.size() > c.d_tlist_cap) {
        if (c.d_tlist) CK(cudaFree(c.d_tlist));
        c.d_tlist_cap = std::max<int>((int)slots.size(), 2 * c.d_tlist_cap);
        CK(cudaMalloc(&c.d_tlist, (size_t)c.d_tlist_cap * sizeof(int)));
    }
    if (!slots.empty()) {
        CK(kg_cpy(c, c.d_tlist, slots.data(), slots.size() * sizeof(int), cudaMemcpyHostToDevice));
        CK(launch_topo32(c.A, c.d_tlist, (int)slots.size(), ts, c.nX, c.nY, c.st));
        c.launches++;
    }
    c.tdirty[ts] = 0;
}

constexpr unsigned long long HUGE_BITS = 0x7FEFFFFFFFFFFFFFull;  // bits of huge(1.0_wp)
// CFL words of the context: the three RK stages of a hydraulic step, and the RHS pass that
// sets or checks dt.
enum { W_S1 = 0, W_S2 = 1, W_S3 = 2, W_RHS = 3 };

int partial(const kg_ctx& c) { return (int)c.active.size() < c.nTiles ? 1 : 0; }

// Queue one fused pass that reduces its CFL terms into word `word` of the context's CFL
// array; nothing waits for it.
void launch_pass(kg_ctx& c, StepArgs& S, int word) {
    S.cfl_min = c.d_cfl + word;
    S.partial = partial(c);
    const bool fp32 = c.prec == KG_PREC_FP32;
    if (fp32 && c.tdirty[S.topo]) refresh_topo32(c, S.topo);
    if (c.timing) CK(cudaEventRecord(c.ev0[word], c.st));
    if (fp32) CK(launch_hydro32(c.A, c.d_blocks, (int)c.blocks.size(), S, c.st));
    else CK(launch_hydro(c.A, c.d_blocks, (int)c.blocks.size(), S, c.st));
    if (c.timing) CK(cudaEventRecord(c.ev1[word], c.st));
    c.launches++;
}
void reset_cfl(kg_ctx& c, int first, int n) {
    for (int k = first; k < first + n; ++k) c.h_cfl[k] = HUGE_BITS;
    CK(kg_cpy(c, c.d_cfl + first, c.h_cfl + first, (size_t)n * sizeof(unsigned long long), cudaMemcpyHostToDevice));
}
// Read back the CFL words (and whatever else was queued for reading) with one wait.
void collect_cfl(kg_ctx& c) {
    CK(kg_cpy(c, c.h_ctl, c.d_ctl, sizeof(kg_ctx::Ctl), cudaMemcpyDeviceToHost));
    sync(c);
}
// Accumulate the event timing of one pass of the last queue (one that ran).
void account_pass(kg_ctx& c, int word) {
    if (!c.timing) return;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c.ev0[word], c.ev1[word]));
    c.kernel_ms += ms;
    c.timed_passes++;
}

unsigned long long run_pass(kg_ctx& c, StepArgs S) {
    reset_cfl(c, W_RHS, 1);
    S.ngate = 0;
    launch_pass(c, S, W_RHS);
    collect_cfl(c);
    account_pass(c, W_RHS);
    return c.h_cfl[W_RHS];
}

double next_flux_time(const kg_ctx& c, double t) {  // NextFluxSeriesTime, src/TimeStepper.f90:281-305
    double nextT = HUGE_D, tdiff = HUGE_D;
    for (const HostSource& s : c.srcs)
        for (int j = 0; j < s.n; ++j) {
            double tmp = s.time[j] - t;
            if (tmp > 0.0 && tmp < tdiff) { tdiff = tmp; nextT = s.time[j]; }
        }
    return nextT;
}

// Queue HydraulicTimeStepper's three stages back to back.  Stage 2 runs only if stage 1's
// advised dt accepts dt and stage 3 only if both do (the test the host applies afterwards
// to the CFL words), so one wait serves the whole step and a refined attempt leaves no
// output behind.  dt comes from the host, or from the device (dtp: the step's first
// attempt, see k_dt).  gflag / gs1 close all three stages: a refine flag that is set, and
// the CFL word of an RHS check whose substep-1 advised dt is below dt.  flags_after queues
// the edge-band flags of the result for the next CheckIfNearBoundaries.
void queue_hydraulic(kg_ctx& c, double dt, const double* dtp, int q_in, int e_set, int topo, int q_s1, int q_s2, int q_out,
                     const int* gflag, const unsigned long long* gs1, bool flags_after) {
    double nextT = c.t + dt;
    StepArgs S{};
    S.q_in = q_in; S.q_s1 = q_s1; S.q_s2 = q_s2; S.q_out = q_out; S.e_set = e_set; S.topo = topo;
    S.q_tc = c.qcur; S.topo_tc = c.tcur;
    // UpdateMaximum* reads the step-start state, so after the first accepted half-step of a
    // step every later one (the second half-step, the half-steps of a retry) finds each
    // maximum already taken with strict comparisons and changes nothing: it is skipped.
    S.dt = dt; S.dtp = dtp; S.t_grid = c.t; S.do_maxima = c.maxima_done ? 0 : 1;
    S.gate_flag = gflag;
    int g0 = 0;
    if (gs1) { S.gate[0] = gs1; S.gate_s1[0] = 1; g0 = 1; }
    reset_cfl(c, W_S1, 3);
    S.mode = MODE_S1; S.t_rhs = nextT; S.tmode = 1; S.ngate = g0;
    launch_pass(c, S, W_S1);
    S.mode = MODE_S2; S.t_rhs = c.t + 0.5 * dt; S.tmode = 2;
    S.gate[g0] = c.d_cfl + W_S1; S.gate_s1[g0] = 0; S.ngate = g0 + 1;
    launch_pass(c, S, W_S2);
    S.mode = MODE_S3; S.t_rhs = nextT; S.t_max = nextT; S.tmode = 1;
    S.gate[g0 + 1] = c.d_cfl + W_S2; S.gate_s1[g0 + 1] = 0; S.ngate = g0 + 2;
    launch_pass(c, S, W_S3);
    if (flags_after) {
        int n = (int)c.active.size(), per = (c.SC + 255) / 256;
        ensure_flags(c, (size_t)n);
        CK(launch_act_flags(c.A, c.d_active, n, q_out, topo, nullptr, c.d_flags, c.nX, c.nY, c.st));
        c.launches++;
        if (n * per > c.h_act_cap) {
            if (c.h_act) CK(cudaFreeHost(c.h_act));
            c.h_act_cap = std::max<int>(n * per, 2 * c.h_act_cap);
            CK(cudaMallocHost(&c.h_act, (size_t)c.h_act_cap * sizeof(int)));
        }
        CK(kg_cpy(c, c.h_act, c.d_flags, (size_t)n * per * sizeof(int), cudaMemcpyDeviceToHost));
    }
}

// The host's refinement tests of HydraulicTimeStepper (src/TimeStepper.f90:393-404,
// :452-463) on the stage CFL words after the wait; true (and the refined dt) on rejection.
bool finish_hydraulic(kg_ctx& c, double& dt, int q_out, int topo, bool flags_after, const int* chunks = nullptr) {
    double dt1 = advised(c, c.h_cfl[W_S1], 2);
    if (dt1 < dt) { account_pass(c, W_S1); dt = 0.9 * dt1; return true; }
    double dt2 = advised(c, c.h_cfl[W_S2], 3);
    if (dt2 < dt) { account_pass(c, W_S1); account_pass(c, W_S2); dt = 0.9 * dt2; return true; }
    account_pass(c, W_S1); account_pass(c, W_S2); account_pass(c, W_S3);
    if (flags_after) {
        int n = (int)c.active.size(), per = (c.SC + 255) / 256;
        c.act_flags.assign((size_t)n, 0);
        for (int q = 0; q < n; ++q)
            for (int k = 0; k < per; ++k) c.act_flags[(size_t)q] |= (chunks ? chunks : c.h_act)[q * per + k];
        c.act_q = q_out;
        c.act_t = topo;
        c.act_gen = c.gen;
    }
    return false;
}


// CalculateHydraulicRHS at substep 1 on state q_in / topography topo into E/I set e_set.
StepArgs rhs_args(const kg_ctx& c, int q_in, int e_set, int topo, double t) {
    StepArgs S{};
    S.mode = MODE_RHS0; S.q_in = q_in; S.e_set = e_set; S.topo = topo; S.t_rhs = t; S.t_grid = c.t;
    S.q_tc = c.qcur; S.topo_tc = c.tcur;
    return S;
}
double rhs0(kg_ctx& c, int q_in, int e_set, int topo, double t, int substep = 1) {
    return advised(c, run_pass(c, rhs_args(c, q_in, e_set, topo, t)), substep);
}

// Dependency waves of the ordered redistribution list (see k_m_redist): candidate q goes
// to wave 1 + the largest wave among the earlier candidates whose cell lies within 2 cells
// of its own (with wrap-around on periodic domains).  The lists come back grouped by wave,
// list order kept inside each wave; woff holds the wave offsets.
void redistribution_waves(kg_ctx& c, const std::vector<int>& slots, const std::vector<unsigned long long>& key,
                          const std::vector<int>& ord, std::vector<int>& ls, std::vector<int>& lc, std::vector<int>& woff) {
    const int n = (int)ord.size();
    const long long NXc = (long long)c.p.nXtiles * c.nX, NYc = (long long)c.p.nYtiles * c.nY;
    const bool per = c.p.bcs == KG_BC_PERIODIC;
    std::vector<long long> gx((size_t)n), gy((size_t)n);
    std::vector<int> qs((size_t)n), qc((size_t)n);
    for (int q = 0; q < n; ++q) {
        unsigned long long k = key[(size_t)ord[(size_t)q]];
        int s = slots[(size_t)(k >> 32)], cell = (int)(k & 0xffffffffull);
        int id = c.slot_tile[(size_t)s];
        qs[(size_t)q] = s;
        qc[(size_t)q] = cell;
        gx[(size_t)q] = (long long)((id - 1) % c.p.nXtiles) * c.nX + cell % c.nX;
        gy[(size_t)q] = (long long)((id - 1) / c.p.nXtiles) * c.nY + cell / c.nX;
    }
    // Wave of the latest candidate per cell, kept per tile (tables are allocated the first
    // time a tile holds a candidate and are cleared again before returning).
    auto& tab = c.redist_grid;
    if (tab.size() != (size_t)c.p.nXtiles * c.p.nYtiles) tab.assign((size_t)c.p.nXtiles * c.p.nYtiles, std::vector<int>());
    auto at = [&](long long x, long long y, bool make) -> int* {
        if (per) { x = (x % NXc + NXc) % NXc; y = (y % NYc + NYc) % NYc; }
        if (x < 0 || x >= NXc || y < 0 || y >= NYc) return nullptr;
        std::vector<int>& t = tab[(size_t)((y / c.nY) * c.p.nXtiles + x / c.nX)];
        if (t.empty()) {
            if (!make) return nullptr;
            t.assign((size_t)c.nX * c.nY, 0);
        }
        return &t[(size_t)((y % c.nY) * c.nX + x % c.nX)];
    };
    std::vector<int> wave((size_t)n);
    int nw = 0;
    for (int q = 0; q < n; ++q) {
        int m = 0;
        for (int dy = -2; dy <= 2; ++dy)
            for (int dx = -2; dx <= 2; ++dx) {
                const int* v = at(gx[(size_t)q] + dx, gy[(size_t)q] + dy, false);
                if (v) m = std::max(m, *v);
            }
        wave[(size_t)q] = m + 1;
        *at(gx[(size_t)q], gy[(size_t)q], true) = m + 1;
        nw = std::max(nw, m + 1);
    }
    for (int q = 0; q < n; ++q) *at(gx[(size_t)q], gy[(size_t)q], true) = 0;
    woff.assign((size_t)nw + 1, 0);
    for (int q = 0; q < n; ++q) woff[(size_t)wave[(size_t)q]]++;
    for (int w = 1; w <= nw; ++w) woff[(size_t)w] += woff[(size_t)w - 1];
    std::vector<int> fill(woff.begin(), woff.end() - 1);
    ls.assign((size_t)n, 0);
    lc.assign((size_t)n, 0);
    for (int q = 0; q < n; ++q) {
        int at = fill[(size_t)wave[(size_t)q] - 1]++;
        ls[(size_t)at] = qs[(size_t)q];
        lc[(size_t)at] = qc[(size_t)q];
    }
}

// The Strang remainder M(2 dt) H(dt) of a step whose first H(dt) was accepted
// (src/TimeStepper.f90:193-270): MorphodynamicTimeStepper (:532-781) on o[0], building the
// new bed in set tnew, then the RHS check of the M result at t0 + dt and the second
// HydraulicTimeStepper into o[1].  Waits: after the M checks (plus one to read the
// redistribution list when there is one) and one at the end; the RHS check and the
// second H are gated on the device by the redistribution's refine flag and the check's
// advised dt.  Returns 0 accepted, 1 M refined, 2 the check cut dt, 3 H refined; dt is
// updated as the reference updates it.
// Queues M on the first hydraulic half-step's result o[0]: init, the three stages, the
// check and the read-back of the leading candidates, ready for one wait.  dtp: the
// half-step's dt on the device (an M queued behind the first attempt of a step, before the
// host has read that dt), else dt.  M writes only the scratch topography set, the M state
// and the candidate list, so an M queued behind a half-step that is then refused is
// simply discarded.
void queue_morpho(kg_ctx& c, double dt, const double* dtp, const int o[3], int tnew) {
    const int qa = o[0];
    double dt_m = 2.0 * dt;
    int n = (int)c.active.size();
    const int* dl = c.d_active;
    const bool fp32 = c.prec == KG_PREC_FP32;
    // The FP32 form's M kernels read gamma of the step-start topography from the cache.
    if (fp32 && c.tdirty[c.tcur]) refresh_topo32(c, c.tcur);
    int need = n * c.SC;
    if (need > c.cand_cap) {
        CK(cudaStreamSynchronize(c.st));
        cudaFree(c.d_ckey); cudaFree(c.d_cex); cudaFree(c.d_rslot); cudaFree(c.d_rcell); cudaFree(c.d_rwave);
        c.cand_cap = std::max(need, 2 * c.cand_cap);
        CK(cudaMalloc(&c.d_ckey, (size_t)c.cand_cap * sizeof(unsigned long long)));
        CK(cudaMalloc(&c.d_cex, (size_t)c.cand_cap * sizeof(double)));
        CK(cudaMalloc(&c.d_rslot, (size_t)c.cand_cap * sizeof(int)));
        CK(cudaMalloc(&c.d_rcell, (size_t)c.cand_cap * sizeof(int)));
        CK(cudaMalloc(&c.d_rwave, ((size_t)c.cand_cap + 1) * sizeof(int)));
    }
    if (fp32 && c.fused_m && m_stage32_blocks(c.nX, c.nY) > 0) {
        // the FP32 form: init, then one launch per stage, the tests in the third
        CK(launch_m_fused32(c.A, dl, n, c.nX, c.nY, qa, c.tcur, tnew, dt_m, dtp, c.d_mflags, c.d_ckey, c.d_cex, c.d_ncand,
                            c.cand_cap, c.st));
        c.launches += 4;
    } else {
        CK(launch_m_init(c.A, dl, n, c.SV, qa, c.tcur, tnew, c.d_mflags, fp32, c.st));
        c.launches++;
        for (int stage = 1; stage <= 3; ++stage) {
            CK(launch_m_emd(c.A, dl, n, c.SC, tnew, fp32, c.st));
            CK(launch_m_bt(c.A, dl, n, c.SV, c.tcur, tnew, stage, dt_m, dtp, fp32, c.st));
            CK(launch_m_cells(c.A, dl, n, c.SC, qa, c.tcur, tnew, fp32, c.st));
            c.launches += 3;
        }
        CK(launch_m_check(c.A, dl, n, c.SC, qa, c.tcur, tnew, c.d_mflags, c.d_ckey, c.d_cex, c.d_ncand, c.cand_cap, fp32, c.st));
        c.launches++;
    }
    int pre = std::min(c.cand_pre, c.cand_cap);
    if (pre > c.h_cand_cap) {
        CK(cudaStreamSynchronize(c.st));
        if (c.h_ckey) CK(cudaFreeHost(c.h_ckey));
        if (c.h_cex) CK(cudaFreeHost(c.h_cex));
        c.h_cand_cap = std::max(pre, 2 * c.h_cand_cap);
        CK(cudaMallocHost(&c.h_ckey, (size_t)c.h_cand_cap * sizeof(unsigned long long)));
        CK(cudaMallocHost(&c.h_cex, (size_t)c.h_cand_cap * sizeof(double)));
    }
    if (pre > 0) {
        CK(kg_cpy(c, c.h_ckey, c.d_ckey, (size_t)pre * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        CK(kg_cpy(c, c.h_cex, c.d_cex, (size_t)pre * sizeof(double), cudaMemcpyDeviceToHost));
    }
    c.cand_pre_used = pre;
}

// After the wait that follows queue_morpho: the refinement tests, the ordered
// redistribution, the closing launch, the RHS check at t0 + dt and the second half-step.
// Returns 0 when the step is accepted, else the retry code with dt refined.
int finish_morpho_and_h2(kg_ctx& c, double& dt, const int o[3], int tnew) {
    const int qa = o[0];
    double dt_m = 2.0 * dt;
    std::vector<int> slots;
    for (int id : c.active) slots.push_back(T(c, id).slot);
    int n = (int)slots.size();
    const int* dl = c.d_active;
    const bool fp32 = c.prec == KG_PREC_FP32;
    const int pre = c.cand_pre_used;
    int ncand = c.h_ctl->ncand;
    c.cand_pre = std::max(256, std::min(1 << 20, 2 * ncand));
    if (c.h_ctl->mflag != 0) {
        dt_m = 0.5 * dt_m;
        dt = 0.5 * dt_m;
        return 1;
    }
    if (ncand > 0) {
        // AddToRedistList keeps the cells ordered by excess deposition, ties in loop order
        // (src/Redistribute.f90:69-101); RedistributeGrid then walks that list.
        std::vector<unsigned long long> key((size_t)ncand);
        std::vector<double> ex((size_t)ncand);
        if (ncand <= pre) {
            std::memcpy(key.data(), c.h_ckey, (size_t)ncand * sizeof(unsigned long long));
            std::memcpy(ex.data(), c.h_cex, (size_t)ncand * sizeof(double));
        } else {
            CK(kg_cpy(c, key.data(), c.d_ckey, (size_t)ncand * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
            CK(kg_cpy(c, ex.data(), c.d_cex, (size_t)ncand * sizeof(double), cudaMemcpyDeviceToHost));
            sync(c);
        }
        double tp0 = wall();
        std::vector<int> ord((size_t)ncand);
        for (int q = 0; q < ncand; ++q) ord[(size_t)q] = q;
        std::sort(ord.begin(), ord.end(), [&](int a, int b) {
            if (ex[(size_t)a] != ex[(size_t)b]) return ex[(size_t)a] < ex[(size_t)b];
            return key[(size_t)a] < key[(size_t)b];
        });
        std::vector<int> ls, lc, woff;
        redistribution_waves(c, slots, key, ord, ls, lc, woff);
        int nw = (int)woff.size() - 1;
        c.redist_cells += ncand;
        c.redist_waves += nw;
        c.redist_walks++;
        c.host_plan_s += wall() - tp0;
        CK(kg_cpy(c, c.d_rslot, ls.data(), (size_t)ncand * sizeof(int), cudaMemcpyHostToDevice));
        CK(kg_cpy(c, c.d_rcell, lc.data(), (size_t)ncand * sizeof(int), cudaMemcpyHostToDevice));
        CK(kg_cpy(c, c.d_rwave, woff.data(), woff.size() * sizeof(int), cudaMemcpyHostToDevice));
        CK(launch_m_redist(c.A, c.d_rslot, c.d_rcell, c.d_rwave, woff.data(), nw, qa, c.tcur, tnew, c.d_mflags, fp32, c.st));
        c.launches += nw <= KG_REDIST_WAVE_MAX ? nw : 1;
    }
    // Interfacial topography of the new bed and the M result (both scratch until accepted).
    CK(launch_m_close(c.A, dl, n, c.nX, c.nY, qa, tnew, fp32, c.st));
    c.launches++;
    // The fused launch rebuilt the active tiles' factor cache of the new set (FP32 form);
    // ghost tiles' factors are rebuilt by the refresh when they were never built.
    if (fp32) c.tdirty[tnew] = c.tdirty[tnew] > 1 ? 2 : 0;
    else c.tdirty[tnew] = std::max(c.tdirty[tnew], 1);
    // RHS check at t0 + dt, then H(dt) from the M result, gated by both tests.
    c.t = c.t0 + dt;
    StepArgs R = rhs_args(c, o[0], 1, tnew, c.t);
    reset_cfl(c, W_RHS, 1);
    R.ngate = 0;
    launch_pass(c, R, W_RHS);
    c.dt = dt;
    queue_hydraulic(c, dt, nullptr, o[0], 1, tnew, o[1], o[2], o[1], c.d_mflags, c.d_cfl + W_RHS, true);
    collect_cfl(c);
    if (c.h_ctl->mflag != 0) {
        c.t = c.t0;
        dt_m = 0.5 * dt_m;
        dt = 0.5 * dt_m;
        return 1;
    }
    account_pass(c, W_RHS);
    double adv = advised(c, c.h_cfl[W_RHS], 1);
    if (adv < dt) {
        if ((dt - adv) / dt < 0.1) dt = 0.9 * dt;
        else dt = adv;
        c.t = c.t0;
        return 2;
    }
    if (!finish_hydraulic(c, dt, o[1], tnew, true)) return 0;
    c.t = c.t0;
    return 3;
}

// One accepted step of IntegrateTo (src/TimeStepper.f90:151-275): H(dt) alone, or the
// Strang split H(dt) M(2 dt) H(dt) with morphodynamics, retried from the step-start state
// until every part accepts its dt.  The RHS at t, the step's dt (k_dt, on the device) and
// the first attempt of H(dt) are queued together behind one wait.
void integrate_step_body(kg_ctx& c, double tend);
void integrate_step(kg_ctx& c, double tend) {
    double t0 = wall();
    integrate_step_body(c, tend);
    c.host_step_s += wall() - t0;
}
void integrate_step_body(kg_ctx& c, double tend) {
    if (!c.sources_loaded) throw KgError(KG_ERR_STATE, "kg_load_sources must be called before stepping");
    check_near_boundaries(c);
    rebuild_blocks(c);
    const bool morpho = c.p.MorphodynamicsOn != 0;
    int o[3], k = 0;
    for (int b = 0; b < 4; ++b)
        if (b != c.qcur) o[k++] = b;
    int tnew = 1 - c.tcur;
    double tmax = mn(tend, next_flux_time(c, c.t));
    double cap = morpho ? 0.5 * (tmax - c.t) : tmax - c.t;
    c.t0 = c.t;
    c.maxima_done = false;
    StepArgs R = rhs_args(c, c.qcur, 0, c.tcur, c.t);
    reset_cfl(c, W_RHS, 1);
    launch_pass(c, R, W_RHS);
    CK(launch_dt(c.d_cfl + W_RHS, partial(c), cap, c.d_dt, c.st));
    c.launches++;
    queue_hydraulic(c, 0.0, c.d_dt, c.qcur, 0, c.tcur, o[0], o[1], o[0], nullptr, nullptr, !morpho);
    if (morpho) queue_morpho(c, 0.0, c.d_dt, o, tnew);
    collect_cfl(c);
    account_pass(c, W_RHS);
    double adv = mn(advised(c, c.h_cfl[W_RHS], 1), cap);
    double ddt = c.h_ctl->dt;
    if (!(adv == ddt) && !(adv != adv && ddt != ddt))
        throw KgError(KG_ERR_CUDA, "device-side dt differs from the host's");
    c.dt = adv;
    double dt = adv;
    bool first = true;
    int guard = 0, newcur = -1;
    while (true) {
        if (++guard > 100000 || !(dt > 0.0)) throw KgError(KG_ERR_DT, "time step collapsed");
        // Each attempt queues the first hydraulic half-step and, with morphodynamics, M on
        // its result, and waits once for both (the first attempt was queued above with the
        // device-computed dt).
        if (!first) {
            c.dt = dt;
            queue_hydraulic(c, dt, nullptr, c.qcur, 0, c.tcur, o[0], o[1], o[0], nullptr, nullptr, !morpho);
            if (morpho) queue_morpho(c, dt, nullptr, o, tnew);
            collect_cfl(c);
        }
        first = false;
        bool rej = finish_hydraulic(c, dt, o[0], c.tcur, !morpho);
        if (rej) { c.rejected++; continue; }
        c.maxima_done = true;
        if (!morpho) { newcur = o[0]; break; }
        int r = finish_morpho_and_h2(c, dt, o, tnew);
        if (r == 0) { newcur = o[1]; break; }
        c.rejected++;
        c.dt = dt;
    }
    c.qcur = newcur;
    if (morpho) c.tcur = tnew;
    c.t = morpho ? c.t0 + 2.0 * dt : c.t0 + dt;
    c.dt = dt;
    c.steps++;
    c.cell_updates += (int64_t)c.active.size() * c.SC * (morpho ? 2 : 1);
    c.src_override = false;
}

// ---------------------------------------------------------------- sources
// LoadSourceConditions, src/SetSources.f90:47-405 (2D).  Tiles are activated in the
// reference's loop order; the cap/cube increments are then applied to the cells in the
// same order, which gives the same state (activation only touches the new tile).
struct CellMod { int id, ii, jj, kind, idx; double R2; };

void upload_sources(kg_ctx& c);
void load_sources(kg_ctx& c) {
    for (auto& s : c.srcs) s.ncells = 0;
    std::vector<CellMod> mods;
    const kg_params& P = c.p;
    // Bounding boxes to skip tiles far from every cap / cube / source.
    auto near = [&](double xmin, double xmax, double ymin, double ymax) {
        for (int k = 0; k < P.nCaps; ++k) {
            const kg_cap& C = P.caps[k];
            if (C.x + C.radius >= xmin && C.x - C.radius <= xmax && C.y + C.radius >= ymin && C.y - C.radius <= ymax) return true;
        }
        for (int k = 0; k < P.nCubes; ++k) {
            const kg_cube& C = P.cubes[k];
            if (C.x + 0.5 * C.length >= xmin && C.x - 0.5 * C.length <= xmax && C.y + 0.5 * C.width >= ymin &&
                C.y - 0.5 * C.width <= ymax)
                return true;
        }
        for (auto& s : c.srcs)
            if (s.x + s.R >= xmin && s.x - s.R <= xmax && s.y + s.R >= ymin && s.y - s.R <= ymax) return true;
        return false;
    };
    for (int i = 1; i <= c.nXt; ++i)
        for (int j = 1; j <= c.nYt; ++j) {
            int k = tile_id(c, i, j);
            double x0 = cell_x(c, i, 1) - c.dp.dx, x1 = cell_x(c, i, c.nX) + c.dp.dx;
            double y0 = cell_y(c, j, 1) - c.dp.dy, y1 = cell_y(c, j, c.nY) + c.dp.dy;
            if (!near(x0, x1, y0, y1)) continue;
            for (int ii = 1; ii <= c.nX; ++ii)
                for (int jj = 1; jj <= c.nY; ++jj) {
                    double x = cell_x(c, i, ii), y = cell_y(c, j, jj);
                    for (int kk = 0; kk < P.nCaps; ++kk) {
                        const kg_cap& C = P.caps[kk];
                        double R2 = (x - C.x) * (x - C.x) + (y - C.y) * (y - C.y);
                        if (R2 <= C.radius * C.radius) {
                            if (!T(c, k).on) add_tile(c, k);
                            if (T(c, k).on) mods.push_back(CellMod{k, ii, jj, 0, kk, R2});
                        }
                    }
                    for (int kk = 0; kk < P.nCubes; ++kk) {
                        const kg_cube& C = P.cubes[kk];
                        if ((std::fabs(x - C.x) <= 0.5 * C.length) && (std::fabs(y - C.y) <= 0.5 * C.width)) {
                            if (!T(c, k).on) add_tile(c, k);
                            if (T(c, k).on) mods.push_back(CellMod{k, ii, jj, 1, kk, 0.0});
                        }
                    }
                    for (size_t kk = 0; kk < c.srcs.size(); ++kk) {
                        HostSource& S = c.srcs[kk];
                        double R2 = (x - S.x) * (x - S.x) + (y - S.y) * (y - S.y);
                        if (R2 <= S.R * S.R) {
                            if (!T(c, k).on) add_tile(c, k);
                            T(c, k).src = true;
                            S.ncells = S.ncells + 1;
                        }
                    }
                }
        }
    // Apply the cap/cube increments on the host copies of the touched tiles.
    std::vector<int> touched;
    for (auto& m : mods)
        if (!in_list(touched, m.id)) touched.push_back(m.id);
    int SC = c.SC;
    struct Buf { std::vector<double> q, ct, hn, rho, hmax; };
    std::vector<Buf> bufs(touched.size());
    for (size_t q = 0; q < touched.size(); ++q) {
        int s = T(c, touched[q]).slot;
        bufs[q].q.resize((size_t)4 * SC);
        bufs[q].ct.resize((size_t)4 * SC);
        bufs[q].hn.assign((size_t)SC, 0.0);
        bufs[q].rho.assign((size_t)SC, c.p.rhow);
        bufs[q].hmax.resize((size_t)SC);
        CK(kg_cpy(c, bufs[q].hmax.data(), c.A.MX + (size_t)s * 11 * SC, (size_t)SC * sizeof(double), cudaMemcpyDeviceToHost));
        CK(kg_cpy(c, bufs[q].q.data(), c.A.Q[c.qcur] + (size_t)s * 4 * SC, (size_t)4 * SC * sizeof(double), cudaMemcpyDeviceToHost));
        CK(kg_cpy(c, bufs[q].ct.data(), c.A.CT[c.tcur] + (size_t)s * 4 * SC, (size_t)4 * SC * sizeof(double), cudaMemcpyDeviceToHost));
    }
    sync(c);
    for (auto& B : bufs) unpack_state(c, B.q.data(), B.q.data());
    double rhow = c.p.rhow, rhos = c.p.rhos;
    for (auto& m : mods) {
        size_t q = std::find(touched.begin(), touched.end(), m.id) - touched.begin();
        Buf& B = bufs[q];
        size_t cc = (size_t)(m.jj - 1) * c.nX + (m.ii - 1);
        double* w = &B.q[cc];
        double* m1 = &B.q[SC + cc];
        double* m2 = &B.q[2 * (size_t)SC + cc];
        double* hp = &B.q[3 * (size_t)SC + cc];
        double b0c = B.ct[cc], dbx = B.ct[2 * (size_t)SC + cc], dby = B.ct[3 * (size_t)SC + cc];
        double gam = gam_of(c.dp.geo, dbx, dby);
        double Hn_orig = B.hn[cc], rho_orig = B.rho[cc];
        if (m.kind == 0) {
            const kg_cap& C = P.caps[m.idx];
            double rho = rhow + (rhos - rhow) * C.psi;
            double Hn = C.height;
            if (C.shape == KG_SHAPE_FLAT) {
                *w = *w + C.height / gam;
                B.hn[cc] = B.hn[cc] + C.height;
                B.hmax[cc] = B.hmax[cc] + C.height;
                *m1 = *m1 + rho * C.height * C.u;
                *m2 = *m2 + rho * C.height * C.v;
                *hp = *hp + C.psi * C.height;
            } else if (C.shape == KG_SHAPE_PARA) {
                double f = C.height * (1.0 - m.R2 / C.radius / C.radius);
                *w = *w + f / gam;
                B.hn[cc] = B.hn[cc] + f;
                B.hmax[cc] = B.hmax[cc] + f;
                *m1 = *m1 + rho * C.height * C.u;
                *m2 = *m2 + rho * C.height * C.v;
                *hp = *hp + C.psi * C.height * (1.0 - m.R2 / C.radius / C.radius);
            } else {
                double hpv = C.height - b0c;
                Hn = hpv * gam;
                if (Hn > 0.0) {
                    *w = *w + hpv;
                    B.hn[cc] = B.hn[cc] + Hn;
                    B.hmax[cc] = B.hmax[cc] + Hn;
                    *m1 = *m1 + rho * Hn * C.u;
                    *m2 = *m2 + rho * Hn * C.v;
                    *hp = *hp + C.psi * Hn;
                }
            }
            B.rho[cc] = (rho_orig * Hn_orig + rho * Hn) / (Hn_orig + Hn);
        } else {
            const kg_cube& C = P.cubes[m.idx];
            double rho = rhow + (rhos - rhow) * C.psi;
            double Hn = C.height;
            if (C.shape == KG_SHAPE_LEVEL) {
                double hpv = C.height - b0c;
                Hn = hpv * gam;
                if (Hn > 0.0) {
                    *w = *w + hpv;
                    B.hn[cc] = B.hn[cc] + Hn;
                    B.hmax[cc] = B.hmax[cc] + Hn;
                    *hp = *hp + Hn * C.psi;
                    *m1 = *m1 + 0.0;
                    *m2 = *m2 + 0.0;
                }
            } else {
                *w = *w + C.height / gam;
                B.hn[cc] = B.hn[cc] + C.height;
                B.hmax[cc] = B.hmax[cc] + C.height;
                *m1 = *m1 + 0.0;
                *m2 = *m2 + 0.0;
                *hp = *hp + C.psi * C.height;
            }
            B.rho[cc] = (rho_orig * Hn_orig + rho * Hn) / (Hn_orig + Hn);
        }
    }
    // Depth/density as the reference holds them after the sources: activation leaves
    // Hn = 0 and rho = rhow everywhere, the cap/cube loops then overwrite cells.
    {
        std::vector<double> z((size_t)SC, 0.0), r((size_t)SC, rhow);
        for (int id : c.active) {
            int s = T(c, id).slot;
            CK(kg_cpy(c, c.d_srcHn + (size_t)s * SC, z.data(), (size_t)SC * sizeof(double), cudaMemcpyHostToDevice));
            CK(kg_cpy(c, c.d_srcRho + (size_t)s * SC, r.data(), (size_t)SC * sizeof(double), cudaMemcpyHostToDevice));
        }
        sync(c);
    }
    for (size_t q = 0; q < touched.size(); ++q) {
        int s = T(c, touched[q]).slot;
        pack_state(c, bufs[q].q.data(), bufs[q].q.data());
        CK(kg_cpy(c, c.A.Q[c.qcur] + (size_t)s * 4 * SC, bufs[q].q.data(), (size_t)4 * SC * sizeof(double), cudaMemcpyHostToDevice));
        CK(kg_cpy(c, c.d_srcHn + (size_t)s * SC, bufs[q].hn.data(), (size_t)SC * sizeof(double), cudaMemcpyHostToDevice));
        CK(kg_cpy(c, c.d_srcRho + (size_t)s * SC, bufs[q].rho.data(), (size_t)SC * sizeof(double), cudaMemcpyHostToDevice));
        CK(kg_cpy(c, c.A.MX + (size_t)s * 11 * SC, bufs[q].hmax.data(), (size_t)SC * sizeof(double), cudaMemcpyHostToDevice));
    }
    sync(c);
    upload_sources(c);
    for (int g : std::vector<int>(c.ghost)) ghost_edges(c, g);
    if (!c.touched.empty()) mirror_touched(c);
    c.src_override = true;
    c.sources_loaded = true;
    c.blocks_dirty = true;
}

// containsSource flags, the per-source cell counts and the device source table.
void upload_sources(kg_ctx& c) {
    for (int id : c.active) {
        int8_t f = T(c, id).src ? 1 : 0;
        CK(kg_cpy(c, c.A.has_source + T(c, id).slot, &f, 1, cudaMemcpyHostToDevice));
        sync(c);
    }
    std::vector<DevSource> ds(c.srcs.size());
    for (size_t k = 0; k < c.srcs.size(); ++k) {
        DevSource& d = ds[k];
        std::memset(&d, 0, sizeof(d));
        d.x = c.srcs[k].x; d.y = c.srcs[k].y; d.R = c.srcs[k].R; d.n = c.srcs[k].n; d.ncells = c.srcs[k].ncells;
        for (int q = 0; q < d.n; ++q) { d.time[q] = c.srcs[k].time[q]; d.flux[q] = c.srcs[k].flux[q]; d.psi[q] = c.srcs[k].psi[q]; }
    }
    c.dsrc = ds;
    if (!ds.empty()) {
        CK(cudaMalloc(&c.d_src, ds.size() * sizeof(DevSource)));
        CK(kg_cpy(c, c.d_src, ds.data(), ds.size() * sizeof(DevSource), cudaMemcpyHostToDevice));
    }
    wait_const_owner(c);
    CK(set_constants(c.dp, ds.data(), (int)ds.size(), c.st));
    g_const_owner = &c;
    sync(c);
}

// LoadInitialCondition_txt + ActivateTile(restart) (src/Restart.f90:151-328,
// src/UpdateTiles.f90:342-384): activate the listed tiles in order, then overwrite their
// conserved fields (w, rhoHnu, rhoHnv, Hnpsi) and their vertex bt, and rebuild what the
// reference rebuilds: cell and interfacial topography, the ghost tiles' edge data and the
// flux-source cell counts (<=, src/Restart.f90:284-305).  The maxima start afresh.
void load_state(kg_ctx& c, const int32_t* ids, int n, const double* state, const double* btv, double t) {
    if (c.sources_loaded) throw KgError(KG_ERR_STATE, "kg_load_state needs a context with nothing loaded");
    for (int k = 0; k < n; ++k) {
        if (!in_bounds(c, ids[k])) throw KgError(KG_ERR_PARAM, "tile id out of range");
        if (!T(c, ids[k]).on) add_tile(c, ids[k]);
    }
    int SC = c.SC, SV = c.SV;
    std::vector<int> slots;
    std::vector<double> packed((size_t)n * 4 * SC);
    for (int k = 0; k < n; ++k) {
        int s = T(c, ids[k]).slot;
        slots.push_back(s);
        double* pk = packed.data() + (size_t)k * 4 * SC;
        pack_state(c, state + (size_t)k * 4 * SC, pk);
        CK(kg_cpy(c, c.A.Q[c.qcur] + (size_t)s * 4 * SC, pk, (size_t)4 * SC * sizeof(double), cudaMemcpyHostToDevice));
        if (btv)
            CK(kg_cpy(c, c.A.BV[c.tcur] + ((size_t)s * 2 + 1) * SV, btv + (size_t)k * SV, (size_t)SV * sizeof(double),
                               cudaMemcpyHostToDevice));
        touch(c, s);
    }
    sync(c);
    upload_list(c, slots);
    CK(launch_cell_topo(c.A, c.d_list, n, c.tcur, c.st));
    CK(launch_face_topo(c.A, c.d_list, n, c.tcur, c.nX, c.nY, false, c.st));
    CK(launch_face_bI(c.A, c.d_list, n, c.tcur, c.nX, c.nY, c.st));
    c.launches += 3;
    sync(c);
    for (auto& src : c.srcs) src.ncells = 0;
    for (int id : c.active) {
        int gi = tile_col(c, id), gj = tile_row(c, id);
        for (int jj = 1; jj <= c.nY; ++jj)
            for (int ii = 1; ii <= c.nX; ++ii) {
                double x = cell_x(c, gi, ii), y = cell_y(c, gj, jj);
                for (auto& src : c.srcs) {
                    double R2 = (x - src.x) * (x - src.x) + (y - src.y) * (y - src.y);
                    if (R2 <= src.R * src.R) {
                        src.ncells = src.ncells + 1;
                        T(c, id).src = true;
                    }
                }
            }
    }
    upload_sources(c);
    for (int g : std::vector<int>(c.ghost)) ghost_edges(c, g);
    if (!c.touched.empty()) mirror_touched(c);
    c.t = t;
    c.src_override = false;
    c.sources_loaded = true;
    c.blocks_dirty = true;
    c.gen++;
    c.tdirty[0] = c.tdirty[1] = 2;
}

// Checks of a caller's kg_params before anything is allocated.  The input parser applies
// the reference's own checks of the input file (src/Parameters.f90, src/SolverSettings.f90,
// src/DomainSettings.f90); these keep a struct filled by any C caller inside what the
// kernels index and branch on.
void validate_params(const kg_params& p) {
    auto bad = [](const char* m) { throw KgError(KG_ERR_PARAM, m); };
    auto within = [](int32_t v, int32_t lo, int32_t hi) { return v >= lo && v <= hi; };
    if (p.nYtiles == 1 && p.nYpertile == 1 && p.nXtiles >= 1 && p.nXpertile >= 1)
        throw KgError(KG_ERR_UNSUPPORTED, "1D grids are not implemented");
    if (p.nXtiles < 1 || p.nYtiles < 1 || p.nXpertile < 2 || p.nYpertile < 2)
        bad("nXtiles/nYtiles must be >= 1 and nXpertile/nYpertile >= 2");
    if ((int64_t)p.nXtiles * p.nYtiles > (int64_t)1 << 30 || (int64_t)p.nXpertile * p.nYpertile > (int64_t)1 << 24)
        bad("more than 2^30 tiles or 2^24 cells per tile");
    if (!(p.Xtilesize > 0.0) || !(p.Ytilesize > 0.0) || !std::isfinite(p.Xtilesize) || !std::isfinite(p.Ytilesize))
        bad("Xtilesize and Ytilesize must be positive and finite");
    if (!(p.cfl > 0.0) || !(p.heightThreshold > 0.0) || !(p.maxdt > 0.0))
        bad("cfl, heightThreshold and maxdt must be positive");
    if (p.TileBuffer < 0) bad("TileBuffer must be >= 0");
    if (!within(p.nSources, 0, KG_MAX_SOURCES) || !within(p.nCaps, 0, KG_MAX_CAPS) || !within(p.nCubes, 0, KG_MAX_CUBES))
        bad("nCaps, nCubes and nSources must lie in 0..16");
    for (int k = 0; k < p.nSources; ++k)
        if (!within(p.sources[k].n_series, 1, KG_MAX_SERIES)) bad("bad flux series length");
    if (!within(p.drag, KG_DRAG_CHEZY, KG_DRAG_MANNING) || !within(p.erosion, KG_ERO_OFF, KG_ERO_GRANULAR) ||
        !within(p.deposition, KG_DEP_NONE, KG_DEP_SPEARMAN_MANNING) ||
        !within(p.erosion_transition, KG_ETRANS_SMOOTH, KG_ETRANS_OFF) ||
        !within(p.morpho_damping, KG_DAMP_NONE, KG_DAMP_RAT3) || !within(p.fswitch, KG_SWITCH_TANH, KG_SWITCH_STEP) ||
        !within(p.limiter, KG_LIM_MINMOD1, KG_LIM_NONE) || !within(p.bcs, KG_BC_HALT, KG_BC_SPONGE) ||
        !within(p.topog, KG_TOPO_UPLOAD, KG_TOPO_XTRISLOPE))
        bad("a closure, limiter, boundary or topography selector is out of range");
}

// Run settings (src/DomainSettings.f90:185-225, src/Parameters.f90:629-648).
void setup(kg_ctx& c, const kg_params& p) {
    c.p = p;
    validate_params(p);
    c.nX = p.nXpertile; c.nY = p.nYpertile; c.nXt = p.nXtiles; c.nYt = p.nYtiles; c.nTiles = c.nXt * c.nYt;
    c.SC = c.nX * c.nY; c.SV = (c.nX + 1) * (c.nY + 1); c.SFX = (c.nX + 1) * c.nY; c.SFY = c.nX * (c.nY + 1);
    c.nE = std::max(c.nX, c.nY);
    DevParams& d = c.dp;
    d.nX = c.nX; d.nY = c.nY; d.nXtiles = c.nXt; d.nYtiles = c.nYt;
    c.xSize = c.nXt * p.Xtilesize;
    c.ySize = c.nYt * p.Ytilesize;
    d.xSize = c.xSize; d.ySize = c.ySize;
    d.dx = p.Xtilesize / (double)c.nX;
    d.dy = p.Ytilesize / (double)c.nY;
    d.dxR = 1.0 / d.dx;
    d.dyR = 1.0 / d.dy;
    d.hdxR = 0.5 * d.dxR;
    d.hdyR = 0.5 * d.dyR;
    d.geo = p.geometric_factors != 0; d.morpho = p.MorphodynamicsOn != 0;
    d.drag = p.drag; d.erosion = p.erosion; d.deposition = p.deposition; d.etrans = p.erosion_transition;
    d.damping = p.morpho_damping; d.fswitch = p.fswitch; d.limiter = p.limiter; d.bcs = p.bcs;
    d.TileBuffer = p.TileBuffer; d.nSources = p.nSources;
    d.g = p.g; d.rhow = p.rhow; d.rhos = p.rhos;
    const double visc_w = 1.2e-6;
    d.gred = (p.rhos / p.rhow - 1.0) * p.g;
    double Rep = std::sqrt(p.g * p.SolidDiameter) * p.SolidDiameter / visc_w;
    double R = std::pow(d.gred / visc_w / visc_w, 1.0 / 3.0) * p.SolidDiameter;
    d.ws0 = p.ws0_given ? p.ws0 : visc_w / p.SolidDiameter * (std::sqrt(10.36 * 10.36 + 1.048 * R * R * R) - 10.36);
    d.nsettling = (4.7 + 0.41 * std::pow(Rep, 0.75)) / (1.0 + 0.175 * std::pow(Rep, 0.75));
    d.CriticalShields = 0.3 / (1.0 + 1.2 * R) + 0.055 * (1.0 - std::exp(-0.02 * R));
    d.ChezyCo = p.ChezyCo; d.ManningCo = p.ManningCo; d.CoulombCo = p.CoulombCo;
    d.PMin = p.PouliquenMinSlope; d.PMax = p.PouliquenMaxSlope; d.PInt = p.PouliquenIntermediateSlope;
    d.PBeta = p.PouliquenBeta; d.Ebetastar = p.Edwards2019betastar; d.Ekappa = p.Edwards2019kappa; d.EGamma = p.Edwards2019Gamma;
    d.SwRate = p.VoellmySwitchRate; d.SwValue = p.VoellmySwitchValue;
    d.EroRate = p.EroRate; d.EroRateGranular = p.EroRateGranular; d.EroDepth = p.EroDepth;
    d.EroCriticalHeight = p.EroCriticalHeight; d.BedPorosity = p.BedPorosity;
    d.invSolid = 1.0 / (1.0 - p.BedPorosity);
    d.maxPack = p.maxPack; d.SolidDiameter = p.SolidDiameter; d.nu = p.EddyViscosity; d.hThr = p.heightThreshold;
    d.tan1deg = std::tan(PI_D / 180.0);
    d.SpongeStrength = p.SpongeStrength;
    d.cfl = p.cfl; d.maxdt = p.maxdt;
    d.diffusiveTimeScale = HUGE_D;
    if (p.EddyViscosity > 0.0)
        d.diffusiveTimeScale = mn(d.dx * d.dx / p.EddyViscosity, d.dy * d.dy / p.EddyViscosity);
    int Nout = p.Nout > 0 ? p.Nout : 100;
    c.DeltaT = (p.tend - p.tstart) / (double)Nout;
    for (int k = 0; k < p.nSources; ++k) {
        const kg_flux_source& s = p.sources[k];
        if (s.n_series < 1 || s.n_series > KG_MAX_SERIES) throw KgError(KG_ERR_PARAM, "bad flux series length");
        HostSource h;
        h.x = s.x; h.y = s.y; h.R = s.radius; h.n = s.n_series; h.ncells = 0;
        h.time.assign(s.time, s.time + s.n_series);
        h.flux.assign(s.flux, s.flux + s.n_series);
        h.psi.assign(s.psi, s.psi + s.n_series);
        c.srcs.push_back(h);
    }
    c.tiles.assign((size_t)c.nTiles, TileMeta());
    c.nx1 = (int64_t)c.nXt * c.nX + 1;
    c.ny1 = (int64_t)c.nYt * c.nY + 1;
    c.t = 0.0;
    c.A.nE = c.nE;
    CK(cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking));
    CK(cudaMalloc(&c.d_ctl, sizeof(kg_ctx::Ctl)));
    CK(cudaMemset(c.d_ctl, 0, sizeof(kg_ctx::Ctl)));
    c.d_cfl = c.d_ctl->cfl;
    c.d_dt = &c.d_ctl->dt;
    c.d_mflags = &c.d_ctl->mflag;
    c.d_ncand = &c.d_ctl->ncand;
    CK(cudaMalloc(&c.d_vol, 4 * sizeof(double)));
    CK(cudaMallocHost(&c.h_ctl, sizeof(kg_ctx::Ctl)));
    c.h_cfl = c.h_ctl->cfl;
    wait_const_owner(c);
    CK(set_constants(c.dp, nullptr, 0, c.st));
    g_const_owner = &c;
    sync(c);
}

void free_ctx(kg_ctx* c) {
    if (!c) return;
    if (g_const_owner == c) g_const_owner = nullptr;
    if (c->st) cudaStreamSynchronize(c->st);
    for (int b = 0; b < 4; ++b) cudaFree(c->A.Q[b]);
    for (int b = 0; b < 2; ++b) {
        cudaFree(c->A.E[b]); cudaFree(c->A.I[b]); cudaFree(c->A.CT[b]); cudaFree(c->A.FX[b]); cudaFree(c->A.FY[b]); cudaFree(c->A.BV[b]);
        cudaFree(c->A.TD[b]); cudaFree(c->A.TF[b]); cudaFree(c->A.TFX[b]); cudaFree(c->A.TFY[b]);
    }
    cudaFree(c->d_tlist);
    cudaFree(c->d_gather);
    cudaFree(c->d_rb0);
    void* ptrs[] = {c->A.UV, c->A.MS, c->A.EMD, c->A.B0S, c->A.M0, c->A.MF, c->A.BVA, c->A.G9, c->A.GE, c->A.MX,
                    c->A.nbr, c->A.kind, c->A.has_source, c->A.tile_of_slot, c->d_blocks, c->d_list, c->d_flags,
                    c->d_vol, c->d_srcHn, c->d_srcRho, c->d_ckey, c->d_cex, c->d_src,
                    c->d_rslot, c->d_rcell, c->d_rwave};
    for (void* q : ptrs) cudaFree(q);
    if (c->own_ctl) {
        cudaFree(c->d_ctl);
        if (c->h_ctl) cudaFreeHost(c->h_ctl);
    }
    if (c->h_act) cudaFreeHost(c->h_act);
    if (c->h_ckey) cudaFreeHost(c->h_ckey);
    if (c->h_cex) cudaFreeHost(c->h_cex);
    cudaFree(c->d_active);
    for (int k = 0; k < 4; ++k) {
        if (c->ev0[k]) cudaEventDestroy(c->ev0[k]);
        if (c->ev1[k]) cudaEventDestroy(c->ev1[k]);
    }
    if (c->st && c->own_stream) cudaStreamDestroy(c->st);
    delete c;
}

int fail(kg_ctx* c, const KgError& e) {
    if (c) c->err = e.what();
    return e.code;
}

void fill_stats(kg_ctx* c, kg_step_stats* st, int64_t s0, int64_t r0, int64_t cu0, int64_t l0) {
    if (!st) return;
    st->t = c->t;
    st->dt = c->dt;
    st->steps = c->steps - s0;
    st->rejected = c->rejected - r0;
    st->cell_updates = c->cell_updates - cu0;
    st->n_active = (int32_t)c->active.size();
    st->n_ghost = (int32_t)c->ghost.size();
    st->kernel_launches = c->launches - l0;
}

int active_slot(kg_ctx* c, int id) {
    if (!c || id < 1 || id > c->nTiles || !in_list(c->active, id)) return -1;
    return T(*c, id).slot;
}

std::vector<double> d2h(kg_ctx* c, const double* src, size_t n) {
    std::vector<double> v(n);
    CK(kg_cpy(*c, v.data(), src, n * sizeof(double), cudaMemcpyDeviceToHost));
    sync(*c);
    return v;
}

}  // namespace

// Every entry point that touches the device holds the API lock and binds its settings.
#define KG_ENTER(c)                                         \
    std::lock_guard<std::recursive_mutex> kg_lock_(g_api_mu); \
    if (c) {                                                \
        try {                                               \
            bind_constants(*c);                             \
        } catch (const KgError& e) {                        \
            return fail(c, e);                              \
        }                                                   \
    }

#define KG_GUARD(c, ...)                                    \
    try {                                                   \
        __VA_ARGS__;                                        \
    } catch (const KgError& e) {                            \
        return fail(c, e);                                  \
    } catch (const std::exception& e) {                     \
        if (c) c->err = e.what();                           \
        return KG_ERR_PARAM;                                \
    }

extern "C" {

const char* kg_version(void) { return "kestrel_gb300 1.0 (sm_103a)"; }

int kg_create(const kg_params* params, int32_t precision, kg_ctx** out) {
    if (!params || !out) {
        g_create_err = "kg_create: null params or out";
        return KG_ERR_PARAM;
    }
    std::lock_guard<std::recursive_mutex> lock(g_api_mu);
    *out = nullptr;
    if (precision != KG_PREC_FP64 && precision != KG_PREC_FP32) {
        g_create_err = "precision must be KG_PREC_FP64 or KG_PREC_FP32";
        return KG_ERR_UNSUPPORTED;
    }
    kg_ctx* c = nullptr;
    try {
        validate_params(*params);
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess || n < 1) throw KgError(KG_ERR_CUDA, "no CUDA device is available");
        c = new kg_ctx();
        c->prec = precision;
        setup(*c, *params);
    } catch (const KgError& e) {
        g_create_err = e.what();
        free_ctx(c);
        return e.code;
    } catch (const std::bad_alloc&) {
        g_create_err = "host allocation failed";
        free_ctx(c);
        return KG_ERR_OOM;
    }
    g_create_err.clear();
    *out = c;
    return KG_OK;
}

void kg_destroy(kg_ctx* ctx) {
    std::lock_guard<std::recursive_mutex> lock(g_api_mu);
    free_ctx(ctx);
}

const char* kg_last_error(const kg_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_err.c_str(); }

int kg_upload_b0(kg_ctx* c, const double* b0, int64_t nx1, int64_t ny1) {
    if (!c || !b0) return KG_ERR_PARAM;
    if (nx1 != c->nx1 || ny1 != c->ny1) {
        c->err = "b0 grid must be (nXtiles*nXpertile+1) x (nYtiles*nYpertile+1)";
        return KG_ERR_PARAM;
    }
    c->upload.assign(b0, b0 + nx1 * ny1);
    return KG_OK;
}

// Every tile's vertex heights from the raster, on the GPU (kg_dem.cu), kept on the device
// until the tiles are activated.
void upload_raster(kg_ctx& c, const double* values, const kg_raster& g) {
    RasterGeo G{g.nx, g.ny, g.origin_x, g.origin_y, g.pixel_w, g.pixel_h, g.nodata, g.center_e, g.center_n,
                c.dp.dx, c.dp.dy, c.nX, c.nY, c.nXt, c.nYt};
    std::vector<double> XV((size_t)c.nXt * (c.nX + 1)), YV((size_t)c.nYt * (c.nY + 1));
    for (int gi = 1; gi <= c.nXt; ++gi) vertex_x(c, gi, XV.data() + (size_t)(gi - 1) * (c.nX + 1));
    for (int gj = 1; gj <= c.nYt; ++gj) vertex_y(c, gj, YV.data() + (size_t)(gj - 1) * (c.nY + 1));
    double *dR = nullptr, *dXV = nullptr, *dYV = nullptr;
    int* dst = nullptr;
    size_t nR = (size_t)g.nx * (size_t)g.ny;
    auto release = [&]() { cudaFree(dR); cudaFree(dXV); cudaFree(dYV); cudaFree(dst); };
    try {
        if (!c.d_rb0) CK(cudaMalloc(&c.d_rb0, (size_t)c.nTiles * c.SV * sizeof(double)));
        CK(cudaMalloc(&dR, nR * sizeof(double)));
        CK(cudaMalloc(&dXV, XV.size() * sizeof(double)));
        CK(cudaMalloc(&dYV, YV.size() * sizeof(double)));
        CK(cudaMalloc(&dst, (size_t)c.nTiles * sizeof(int)));
        CK(kg_cpy(c, dR, values, nR * sizeof(double), cudaMemcpyHostToDevice));
        CK(kg_cpy(c, dXV, XV.data(), XV.size() * sizeof(double), cudaMemcpyHostToDevice));
        CK(kg_cpy(c, dYV, YV.data(), YV.size() * sizeof(double), cudaMemcpyHostToDevice));
        CK(launch_raster_heights(dR, G, dXV, dYV, c.d_rb0, dst, c.st));
        c.launches++;
        c.raster_status.assign((size_t)c.nTiles, 0);
        CK(kg_cpy(c, c.raster_status.data(), dst, (size_t)c.nTiles * sizeof(int), cudaMemcpyDeviceToHost));
        sync(c);
    } catch (...) {
        release();
        throw;
    }
    release();
}

int kg_upload_raster(kg_ctx* c, const double* values, const kg_raster* geo) {
    if (!c || !values || !geo) return KG_ERR_PARAM;
    KG_ENTER(c);
    if (c->p.topog != KG_TOPO_RASTER) { c->err = "topog is not RASTER"; return KG_ERR_STATE; }
    if (c->sources_loaded) { c->err = "sources already loaded"; return KG_ERR_STATE; }
    if (geo->nx < 1 || geo->ny < 1 || !(geo->pixel_w > 0.0) || !(geo->pixel_h < 0.0) || !std::isfinite(geo->origin_x) ||
        !std::isfinite(geo->origin_y) || !std::isfinite(geo->pixel_w) || !std::isfinite(geo->pixel_h) ||
        !std::isfinite(geo->center_e) || !std::isfinite(geo->center_n)) {
        c->err = "raster needs nx, ny >= 1, finite georeferencing, pixel_w > 0 and pixel_h < 0 (north-up)";
        return KG_ERR_PARAM;
    }
    KG_GUARD(c, upload_raster(*c, values, *geo));
    return KG_OK;
}

int kg_load_sources(kg_ctx* c) {
    if (!c) return KG_ERR_PARAM;
    KG_ENTER(c);
    if (c->sources_loaded) { c->err = "sources already loaded"; return KG_ERR_STATE; }
    if (c->p.topog == KG_TOPO_UPLOAD && c->upload.empty()) { c->err = "no topography uploaded"; return KG_ERR_STATE; }
    if (c->p.topog == KG_TOPO_RASTER && c->raster_status.empty()) { c->err = "no raster uploaded"; return KG_ERR_STATE; }
    c->gen++;
    KG_GUARD(c, load_sources(*c));
    return KG_OK;
}

int kg_load_state(kg_ctx* c, const int32_t* ids, int32_t n, const double* state, const double* bt_vertex, double t) {
    if (!c || !ids || !state || n < 1) return KG_ERR_PARAM;
    KG_ENTER(c);
    for (int k = 1; k < n; ++k)
        if (ids[k] <= ids[k - 1]) { c->err = "kg_load_state: tile ids must be strictly increasing"; return KG_ERR_PARAM; }
    KG_GUARD(c, load_state(*c, ids, n, state, bt_vertex, t));
    return KG_OK;
}

int kg_step(kg_ctx* c, double t_stop, kg_step_stats* st) {
    if (!c) return KG_ERR_PARAM;
    KG_ENTER(c);
    int64_t s0 = c->steps, r0 = c->rejected, cu0 = c->cell_updates, l0 = c->launches;
    int rc = KG_OK;
    try {
        integrate_step(*c, t_stop);
    } catch (const KgError& e) {
        rc = fail(c, e);
    }
    fill_stats(c, st, s0, r0, cu0, l0);
    return rc;
}

int kg_integrate_to(kg_ctx* c, double t_end, kg_step_stats* st) {
    if (!c) return KG_ERR_PARAM;
    KG_ENTER(c);
    int64_t s0 = c->steps, r0 = c->rejected, cu0 = c->cell_updates, l0 = c->launches;
    int rc = KG_OK;
    if (t_end > c->t) {
        try {
            while (true) {
                integrate_step(*c, t_end);
                if (c->t >= t_end) break;
            }
        } catch (const KgError& e) {
            rc = fail(c, e);
        }
    }
    fill_stats(c, st, s0, r0, cu0, l0);
    return rc;
}

int kg_run(kg_ctx* c, kg_step_stats* st) {
    if (!c) return KG_ERR_PARAM;
    KG_ENTER(c);
    int64_t s0 = c->steps, r0 = c->rejected, cu0 = c->cell_updates, l0 = c->launches;
    int Nout = c->p.Nout > 0 ? c->p.Nout : 100;
    int rc = KG_OK;
    for (int i = 1; i <= Nout && rc == KG_OK; ++i) rc = kg_integrate_to(c, c->p.tstart + i * c->DeltaT, nullptr);
    fill_stats(c, st, s0, r0, cu0, l0);
    return rc;
}

int kg_hydraulic_rhs(kg_ctx* c, double t, int32_t substep, double* advised_dt) {
    if (!c || !advised_dt || substep < 1 || substep > 4) return KG_ERR_PARAM;
    KG_ENTER(c);
    KG_GUARD(c, {
        rebuild_blocks(*c);
        *advised_dt = rhs0(*c, c->qcur, 0, c->tcur, t, substep);
    });
    return KG_OK;
}

int kg_get_active_tiles(kg_ctx* c, int32_t* ids, int32_t* n) {
    if (!c || !n) return KG_ERR_PARAM;
    int cap = *n;
    *n = (int32_t)c->active.size();
    for (int i = 0; ids && i < std::min(cap, *n); ++i) ids[i] = c->active[(size_t)i];
    return KG_OK;
}
int kg_get_ghost_tiles(kg_ctx* c, int32_t* ids, int32_t* n) {
    if (!c || !n) return KG_ERR_PARAM;
    int cap = *n;
    *n = (int32_t)c->ghost.size();
    for (int i = 0; ids && i < std::min(cap, *n); ++i) ids[i] = c->ghost[(size_t)i];
    return KG_OK;
}

int kg_get_tile_field(kg_ctx* c, int32_t id, int32_t field, double* out) {
    if (!c) return KG_ERR_PARAM;
    KG_ENTER(c);
    int s = active_slot(c, id);
    if (s < 0) return KG_ERR_NOT_FOUND;
    if (field < 1 || field > 13 || !out) return KG_ERR_PARAM;
    KG_GUARD(c, {
        int SC = c->SC;
        if ((field == 2 || field == 3) && c->prec == KG_PREC_FP32) {
            auto v = d2h(c, c->A.Q[c->qcur] + ((size_t)s * 4 + 1) * SC, SC);
            const float* m = reinterpret_cast<const float*>(v.data()) + (field == 3 ? SC : 0);
            for (int k = 0; k < SC; ++k) out[k] = (double)m[k];
        } else if (field <= 4) {
            auto v = d2h(c, c->A.Q[c->qcur] + ((size_t)s * 4 + field - 1) * SC, SC);
            std::memcpy(out, v.data(), SC * sizeof(double));
        } else if (field >= 10) {
            auto v = d2h(c, c->A.CT[c->tcur] + ((size_t)s * 4 + field - 10) * SC, SC);
            std::memcpy(out, v.data(), SC * sizeof(double));
        } else if (field == 6 || field == 7) {
            auto v = d2h(c, c->A.UV + ((size_t)s * 2 + field - 6) * SC, SC);
            std::memcpy(out, v.data(), SC * sizeof(double));
        } else {
            auto q = d2h(c, c->A.Q[c->qcur] + (size_t)s * 4 * SC, 4 * (size_t)SC);
            auto ct = d2h(c, c->A.CT[c->tcur] + (size_t)s * 4 * SC, 4 * (size_t)SC);
            std::vector<double> hn, rh;
            if (c->src_override) {
                hn = d2h(c, c->d_srcHn + (size_t)s * SC, SC);
                rh = d2h(c, c->d_srcRho + (size_t)s * SC, SC);
            }
            double e2 = c->dp.hThr * c->dp.hThr;
            for (int k = 0; k < SC; ++k) {
                double gam = gam_of(c->dp.geo, ct[2 * (size_t)SC + k], ct[3 * (size_t)SC + k]);
                double Hn = compute_hn(q[k], ct[k], ct[(size_t)SC + k], gam);
                if (Hn < 0.0) Hn = 0.0;
                double pp = q[3 * (size_t)SC + k] < 0.0 ? 0.0 : q[3 * (size_t)SC + k];
                double psi = mn(2.0 * Hn * pp / (Hn * Hn + mx(Hn * Hn, e2)), c->dp.maxPack);
                double rho = density(c->dp, psi);
                if (c->src_override) { Hn = hn[k]; rho = rh[k]; }
                out[k] = field == 5 ? Hn : field == 8 ? psi : rho;
            }
        }
    });
    return KG_OK;
}

int kg_get_state(kg_ctx* c, int32_t* ids, int32_t* n, double* state, double* bt_vertex) {
    if (!c || !n) return KG_ERR_PARAM;
    KG_ENTER(c);
    const int cap = *n, na = (int)c->active.size();
    *n = (int32_t)na;
    if (!ids && !state && !bt_vertex) return KG_OK;  // the count only
    if (cap < na) {
        c->err = "kg_get_state: room for " + std::to_string(cap) + " tiles, " + std::to_string(na) + " are active";
        return KG_ERR_PARAM;
    }
    for (int k = 0; ids && k < na; ++k) ids[k] = c->active[(size_t)k];
    if ((!state && !bt_vertex) || na == 0) return KG_OK;
    KG_GUARD(c, {
        const size_t SC = (size_t)c->SC, SV = (size_t)c->SV, need = (size_t)na * (4 * SC + SV);
        if (need > c->d_gather_cap) {
            if (c->d_gather) CK(cudaFree(c->d_gather));
            c->d_gather = nullptr;
            c->d_gather_cap = 0;
            CK(cudaMalloc(&c->d_gather, need * sizeof(double)));
            c->d_gather_cap = need;
        }
        std::vector<int> slots;
        for (int id : c->active) slots.push_back(T(*c, id).slot);
        upload_list(*c, slots);
        double* du4 = c->d_gather;
        double* dbt = c->d_gather + (size_t)na * 4 * SC;
        CK(launch_gather_state(c->A, c->d_list, na, c->qcur, c->tcur, (int)SC, (int)SV, c->prec == KG_PREC_FP32, du4, dbt, c->st));
        c->launches++;
        if (state) CK(kg_cpy(*c, state, du4, (size_t)na * 4 * SC * sizeof(double), cudaMemcpyDeviceToHost));
        if (bt_vertex) CK(kg_cpy(*c, bt_vertex, dbt, (size_t)na * SV * sizeof(double), cudaMemcpyDeviceToHost));
        sync(*c);
    });
    return KG_OK;
}

int kg_set_tile_field(kg_ctx* c, int32_t id, int32_t field, const double* in) {
    if (!c) return KG_ERR_PARAM;
    KG_ENTER(c);
    int s = active_slot(c, id);
    if (s < 0) return KG_ERR_NOT_FOUND;
    if (field < 1 || field > 4 || !in) return KG_ERR_PARAM;
    c->gen++;
    KG_GUARD(c, {
        if ((field == 2 || field == 3) && c->prec == KG_PREC_FP32) {
            // the FP32 form's momentum plane holds both momenta as floats
            double* pl = c->A.Q[c->qcur] + ((size_t)s * 4 + 1) * c->SC;
            auto v = d2h(c, pl, (size_t)c->SC);
            float* m = reinterpret_cast<float*>(v.data()) + (field == 3 ? c->SC : 0);
            for (int k = 0; k < c->SC; ++k) m[k] = (float)in[k];
            CK(kg_cpy(*c, pl, v.data(), (size_t)c->SC * sizeof(double), cudaMemcpyHostToDevice));
        } else {
            CK(kg_cpy(*c, c->A.Q[c->qcur] + ((size_t)s * 4 + field - 1) * c->SC, in, (size_t)c->SC * sizeof(double),
                               cudaMemcpyHostToDevice));
        }
        sync(*c);
    });
    return KG_OK;
}

int kg_get_tile_vertex(kg_ctx* c, int32_t id, int32_t which, double* out) {
    if (!c) return KG_ERR_PARAM;
    std::lock_guard<std::recursive_mutex> kg_lock_(g_api_mu);
    int s = active_slot(c, id);
    if (s < 0) return KG_ERR_NOT_FOUND;
    if (which < 0 || which > 1 || !out) return KG_ERR_PARAM;
    KG_GUARD(c, {
        auto v = d2h(c, c->A.BV[c->tcur] + ((size_t)s * 2 + which) * c->SV, c->SV);
        std::memcpy(out, v.data(), (size_t)c->SV * sizeof(double));
    });
    return KG_OK;
}

int kg_get_tile_rhs(kg_ctx* c, int32_t id, int32_t k, double* out) {
    if (!c) return KG_ERR_PARAM;
    std::lock_guard<std::recursive_mutex> kg_lock_(g_api_mu);
    int s = active_slot(c, id);
    if (s < 0) return KG_ERR_NOT_FOUND;
    if (k < 1 || k > 5 || !out) return KG_ERR_PARAM;
    KG_GUARD(c, {
        if (c->prec == KG_PREC_FP32 && (k == 2 || k == 3 || k == 5)) {
            // the FP32 form's momentum rows and ddtImplicit are stored as floats
            const double* src = k == 5 ? c->A.I[0] + (size_t)s * c->SC : c->A.E[0] + ((size_t)s * 4 + 1) * c->SC;
            auto v = d2h(c, src, c->SC);
            const float* f = reinterpret_cast<const float*>(v.data()) + (k == 3 ? c->SC : 0);
            for (int q = 0; q < c->SC; ++q) out[q] = (double)f[q];
        } else {
            const double* src = k <= 4 ? c->A.E[0] + ((size_t)s * 4 + k - 1) * c->SC : c->A.I[0] + (size_t)s * c->SC;
            auto v = d2h(c, src, c->SC);
            std::memcpy(out, v.data(), (size_t)c->SC * sizeof(double));
        }
    });
    return KG_OK;
}

int kg_get_tile_maxima(kg_ctx* c, int32_t id, int32_t which, double* out) {
    if (!c) return KG_ERR_PARAM;
    std::lock_guard<std::recursive_mutex> kg_lock_(g_api_mu);
    int s = active_slot(c, id);
    if (s < 0) return KG_ERR_NOT_FOUND;
    if (which < 0 || which > 5 || !out) return KG_ERR_PARAM;
    KG_GUARD(c, {
        size_t SC = c->SC;
        if (which == 5) {
            auto v = d2h(c, c->A.MX + ((size_t)s * 11 + 10) * SC, SC);
            std::memcpy(out, v.data(), SC * sizeof(double));
        } else {
            auto v = d2h(c, c->A.MX + ((size_t)s * 11 + 2 * which) * SC, 2 * SC);
            std::memcpy(out, v.data(), 2 * SC * sizeof(double));
        }
    });
    return KG_OK;
}

int kg_volume(kg_ctx* c, double out[4]) {
    if (!c || !out) return KG_ERR_PARAM;
    KG_ENTER(c);
    KG_GUARD(c, {
        std::vector<int> slots;
        for (int id : c->active) slots.push_back(T(*c, id).slot);
        upload_list(*c, slots);
        CK(launch_volume(c->A, c->d_list, (int)slots.size(), c->qcur, c->tcur, c->src_override ? c->d_srcHn : nullptr,
                         c->src_override ? c->d_srcRho : nullptr, c->d_vol, c->st));
        c->launches++;
        auto v = d2h(c, c->d_vol, 4);
        for (int k = 0; k < 4; ++k) out[k] = v[k];
    });
    return KG_OK;
}

int kg_get_time(kg_ctx* c, double* t, double* dt) {
    if (!c || !t || !dt) return KG_ERR_PARAM;
    *t = c->t;
    *dt = c->dt;
    return KG_OK;
}

int64_t kg_kernel_launches(const kg_ctx* c) { return c ? c->launches : 0; }

int kg_get_counters(kg_ctx* c, int64_t out[3]) {
    if (!c || !out) return KG_ERR_PARAM;
    out[0] = c->steps;
    out[1] = c->rejected;
    out[2] = c->cell_updates;
    return KG_OK;
}

int kg_get_transfer_bytes(kg_ctx* c, int64_t out[2]) {
    if (!c || !out) return KG_ERR_PARAM;
    out[0] = c->h2d_bytes;
    out[1] = c->d2h_bytes;
    return KG_OK;
}

int64_t kg_device_bytes(kg_ctx* c) {
    if (!c) return 0;
    return (int64_t)bytes_per_slot(*c) * c->cap;
}

int64_t kg_slot_bytes(int32_t nXpertile, int32_t nYpertile, int32_t precision) {
    if (nXpertile < 1 || nYpertile < 1 || (precision != KG_PREC_FP64 && precision != KG_PREC_FP32)) return 0;
    return (int64_t)slot_bytes((size_t)nXpertile, (size_t)nYpertile, precision);
}

int kg_host_times(kg_ctx* c, double out[3]) {
    if (!c || !out) return KG_ERR_PARAM;
    out[0] = c->host_step_s;
    out[1] = c->host_wait_s;
    out[2] = c->host_plan_s;
    return KG_OK;
}

int kg_redistribution_stats(kg_ctx* c, int64_t* cells, int64_t* waves, int64_t* walks) {
    if (!c || !cells || !waves || !walks) return KG_ERR_PARAM;
    *cells = c->redist_cells;
    *waves = c->redist_waves;
    *walks = c->redist_walks;
    return KG_OK;
}

void* kg_stream(kg_ctx* c) { return c ? (void*)c->st : nullptr; }

int kg_set_fused_morpho(kg_ctx* c, int32_t enable) {
    if (!c) return KG_ERR_PARAM;
    c->fused_m = enable != 0;
    return KG_OK;
}

int kg_set_dry_skip(kg_ctx* c, int32_t enable) {
    if (!c) return KG_ERR_PARAM;
    KG_GUARD(c, {
        c->dp.no_dry_skip = enable ? 0 : 1;
        if (g_const_owner == c) g_const_owner = nullptr;  // rewrite the constant bank before the next launch
    });
    return KG_OK;
}

int kg_set_kernel_timing(kg_ctx* c, int32_t enable) {
    if (!c) return KG_ERR_PARAM;
    KG_GUARD(c, {
        if (enable && !c->ev0[0]) {
            for (int k = 0; k < 4; ++k) {
                CK(cudaEventCreate(&c->ev0[k]));
                CK(cudaEventCreate(&c->ev1[k]));
            }
        }
        c->timing = enable != 0;
        c->kernel_ms = 0.0;
        c->timed_passes = 0;
    });
    return KG_OK;
}

int kg_get_kernel_time(kg_ctx* c, double* ms, int64_t* passes) {
    if (!c || !ms || !passes) return KG_ERR_PARAM;
    *ms = c->kernel_ms;
    *passes = c->timed_passes;
    return KG_OK;
}

}  // extern "C"
