// kg_noalloc.cu -- kg_hydraulic_rhs_noalloc: the hydraulic RHS pass without any device
// allocation in the call.
//
// Some hosts own all of the device memory themselves: a Fortran host program that reserves one
// device pool at start-up for its whole run, or a service that admits work against a fixed
// HBM budget, may not let a library call cudaMalloc once it is running.  For them this
// entry point evaluates one CalculateHydraulicRHS on a context created earlier (inputs:
// the context's solution; outputs: its ddtExplicit/ddtImplicit planes and the advised
// time step) and keeps the kernel's scratch -- the CFL-minimum word and the list of tile
// blocks -- in the file-scope array below instead of in context-owned buffers.
//
// Limits and sharing:
//  - The array holds at most KG_NOALLOC_MAX_BLOCKS (65,536) blocks of 16 x 16 cells (about
//    16.7 M active cells); larger active sets are rejected with KG_ERR_PARAM.
//  - The array is about 1 MiB and every GPU that loads the library keeps it until exit.
//  - Every call, on every context of the process, uses the same array.  The CFL word is
//    reset at the start of each call; the block list is rewritten.  Calls that overlap on
//    the GPU (from different host threads or streams) race on it and must not be issued.
//  - The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current).  Make that first
//    call before any stream capture on the device.
#include <cuda_runtime.h>

namespace {

constexpr int KG_NOALLOC_MAX_BLOCKS = 65536;

struct NoAllocScratch {
    unsigned long long cfl_min;           // reduced in the kernel; reset before each launch
    unsigned long long pad[31];           // keeps the block list 256-byte aligned
    kg::BlockDesc blocks[KG_NOALLOC_MAX_BLOCKS];
};

static __device__ __align__(256) NoAllocScratch kg_noalloc_scratch;

// Host-side copy of the array's device address, looked up once per device.  The symbol
// name itself is a host stand-in and must never be handed to a kernel.
constexpr int KG_MAX_DEVICES = 64;
NoAllocScratch* g_scratch_dev[KG_MAX_DEVICES] = {nullptr};

int scratch_for_current_device(NoAllocScratch** out, std::string& err) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= KG_MAX_DEVICES) {
        err = std::string("kg_hydraulic_rhs_noalloc: no current CUDA device: ") + cudaGetErrorString(e);
        return KG_ERR_CUDA;
    }
    if (!g_scratch_dev[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, kg_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            err = std::string("kg_hydraulic_rhs_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
            return KG_ERR_CUDA;
        }
        g_scratch_dev[dev] = static_cast<NoAllocScratch*>(p);
    }
    *out = g_scratch_dev[dev];
    return KG_OK;
}

}  // namespace

extern "C" int kg_hydraulic_rhs_noalloc(kg_ctx* c, double t, int32_t substep, double* advised_dt) {
    if (!c || !advised_dt || substep < 1 || substep > 4) return KG_ERR_PARAM;
    KG_ENTER(c);
    if (c->prec != KG_PREC_FP64) {
        // The FP32 form's factor cache is rebuilt through context-owned scratch.
        c->err = "kg_hydraulic_rhs_noalloc: only FP64 contexts are supported";
        return KG_ERR_UNSUPPORTED;
    }
    if (!c->sources_loaded || c->active.empty()) {
        c->err = "kg_hydraulic_rhs_noalloc: no active tiles (load the sources first)";
        return KG_ERR_STATE;
    }
    NoAllocScratch* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch, c->err);
    if (rc != KG_OK) return rc;
    // The pass reads the neighbour-slot table.  After an activation or a load its corner
    // entries are refreshed only lazily (before the next step); refresh the whole table
    // now, the way the allocating entry point does.  This copies into the table the
    // context already owns and allocates nothing on the device.
    if (c->blocks_dirty) KG_GUARD(c, refresh_all_nbrs(*c));
    // The block list of the active tiles, built on the host exactly as the context's own
    // pass builds it.
    const int BSZ = 16;
    int bx = (c->nX + BSZ - 1) / BSZ, by = (c->nY + BSZ - 1) / BSZ;
    long long nblocks = (long long)c->active.size() * bx * by;
    if (nblocks > KG_NOALLOC_MAX_BLOCKS) {
        c->err = "kg_hydraulic_rhs_noalloc: " + std::to_string(nblocks) + " blocks exceed the static limit of " +
                 std::to_string(KG_NOALLOC_MAX_BLOCKS) + " (16x16-cell blocks)";
        return KG_ERR_PARAM;
    }
    std::vector<kg::BlockDesc> host;
    host.reserve((size_t)nblocks);
    for (int id : c->active) {
        int s = c->tiles[(size_t)id - 1].slot;
        for (int y0 = 0; y0 < c->nY; y0 += BSZ)
            for (int x0 = 0; x0 < c->nX; x0 += BSZ) host.push_back(kg::BlockDesc{s, x0, y0, id});
    }
    unsigned long long huge_bits = 0x7FEFFFFFFFFFFFFFull, bits = 0;
    // Copies go through kg_cpy so that kg_get_transfer_bytes counts them.
    cudaError_t e = kg_cpy(*c, scratch->blocks, host.data(), host.size() * sizeof(kg::BlockDesc), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = kg_cpy(*c, &scratch->cfl_min, &huge_bits, sizeof(huge_bits), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        c->err = std::string("kg_hydraulic_rhs_noalloc: ") + cudaGetErrorString(e);
        return KG_ERR_CUDA;
    }
    kg::StepArgs S{};
    S.mode = kg::MODE_RHS0;
    S.q_in = c->qcur;
    S.e_set = 0;
    S.topo = c->tcur;
    S.q_tc = c->qcur;
    S.topo_tc = c->tcur;
    S.t_rhs = t;
    S.t_grid = c->t;
    S.cfl_min = &scratch->cfl_min;
    e = kg::launch_hydro(c->A, scratch->blocks, (int)host.size(), S, c->st);
    if (e == cudaSuccess) e = kg_cpy(*c, &bits, &scratch->cfl_min, sizeof(bits), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
        c->err = std::string("kg_hydraulic_rhs_noalloc: ") + cudaGetErrorString(e);
        return KG_ERR_CUDA;
    }
    c->launches++;
    *advised_dt = advised(*c, bits, substep);
    return KG_OK;
}
