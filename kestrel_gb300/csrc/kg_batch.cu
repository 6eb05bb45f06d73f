#include <functional>
// kg_batch.cu -- many simulations advanced together (the batched ensemble form).
//
// A batch owns FP32-form simulations of any grid and tile size on one CUDA stream.
// kg_batch_step advances every live member by one round of its current step of
// IntegrateTo (src/TimeStepper.f90:151-275).  The hydraulic passes of all members that are at the
// same stage run as ONE persistent launch over the packed list of their tile blocks
// (k_hydro32_batch: each CTA walks the list with a grid stride and finds its member by a
// binary search of the block offsets); the step's dt selection and the edge-band flags are
// batched the same way, and every wait serves all members at once.  Each member keeps its
// own context (arrays, tiles, dt control, refinement history): its settings come from a
// per-member table instead of the constant bank, and its arithmetic is the single
// simulation's, so a member's results are identical alone and in any mix.
//
// Steps are driven phase by phase:
//   prepare   per member: CheckIfNearBoundaries, block list, step targets
//   H         batched: RHS at t + device dt (fresh steps), the three RK stages (fresh steps
//             and refined retries), edge-band flags; one wait; the host's tests per member
//   M         per member: the morphodynamic operator up to its checks (per-member
//             launches, no wait in between); one wait; redistribution where listed; then
//             batched: the RHS check and the second H, gated on the device; one wait
// until every member has accepted its step.

namespace kg {

// Per-member settings and device lists the batched kernels read.
struct SimStatic {
    DevArrays A;
    DevParams P;
    DevParams32 F;
    const DevSource* src;
    const BlockDesc* blocks;
    const int* slots;  // active slots in list order
    int nblocks, nactive;
};

__global__ void __launch_bounds__(NT) k_hydro32_batch(const SimStatic* __restrict__ sims, const StepArgs* __restrict__ args,
                                                      const int* __restrict__ member, const int* __restrict__ prefix,
                                                      int njobs, int total) {
    kg_dep_wait();
    extern __shared__ __align__(16) unsigned char smraw[];
    Hydro32Smem& sm = *reinterpret_cast<Hydro32Smem*>(smraw);
    for (int b = blockIdx.x; b < total; b += gridDim.x) {
        int lo = 0, hi = njobs - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (prefix[mid] <= b) lo = mid;
            else hi = mid - 1;
        }
        const SimStatic& X = sims[member[lo]];
        const StepArgs& S = args[lo];
        StageTimes Tm;
        if (stage_gate_open_warp(X.P, S, Tm)) hydro32_block(X.A, S, Tm, X.P, X.F, X.src, X.blocks[b - prefix[lo]], sm);
        __syncthreads();
    }
}

// The first dt of a step for each listed member (k_dt's rule with the member's settings).
struct DtJob {
    const unsigned long long* cfl;
    double* dtp;
    double cap;
    int partial, member;
};
__global__ void k_dt_batch(const SimStatic* __restrict__ sims, const DtJob* __restrict__ jobs, int n) {
    kg_dep_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DtJob& J = jobs[i];
    double adv = 0.9 * advised_m(sims[J.member].P, *J.cfl, J.partial);
    *J.dtp = mn(adv, J.cap);
}

// Edge-band flags of each listed member's candidate result, one word per (tile, chunk) at
// out + prefix[job].
struct ActJob {
    int member, q, topo, per;
};
__global__ void __launch_bounds__(256) k_act_flags_batch(const SimStatic* __restrict__ sims, const ActJob* __restrict__ jobs,
                                                          const int* __restrict__ prefix, int njobs, int total, int* out) {
    kg_dep_wait();
    for (int b = blockIdx.x; b < total; b += gridDim.x) {
        int lo = 0, hi = njobs - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (prefix[mid] <= b) lo = mid;
            else hi = mid - 1;
        }
        const ActJob& J = jobs[lo];
        const SimStatic& X = sims[J.member];
        int local = b - prefix[lo];
        int f = block_or(act_bits(X.P, X.A, X.slots[local / J.per], J.q, J.topo, nullptr, local % J.per));
        if (threadIdx.x == 0) out[b] = f;
        __syncthreads();
    }
}

// The morphodynamic operator's per-tile steps for many members in one launch each: job j
// covers member jobs[j].member's active tiles with `per` CTAs per tile (enough for its
// vertices, cells and faces); each CTA runs the same per-item body the single-simulation
// kernel runs, with the member's settings.
struct MJob {
    int member, per, qa, tcur, tnew, cap;
    double dt;
    int* flags;  // the member's M refine flag; the candidate count follows it
    unsigned long long* keys;
    double* ex;
};
enum MKind { MK_INIT, MK_EMD, MK_BT, MK_CELLS, MK_CHECK, MK_CLOSE };

template <int K>
__global__ void __launch_bounds__(256) k_m_batch(const SimStatic* __restrict__ sims, const MJob* __restrict__ jobs,
                                                 const int* __restrict__ prefix, int njobs, int total, int stage) {
    kg_dep_wait();
    for (int b = blockIdx.x; b < total; b += gridDim.x) {
        int lo = 0, hi = njobs - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (prefix[mid] <= b) lo = mid;
            else hi = mid - 1;
        }
        const MJob& J = jobs[lo];
        const SimStatic& X = sims[J.member];
        int local = b - prefix[lo], pos = local / J.per, item = (local % J.per) * 256 + threadIdx.x;
        int s = X.slots[pos];
        if (K == MK_INIT) {
            if (local == 0 && threadIdx.x < 2) J.flags[threadIdx.x] = 0;
            m_init<true>(X.P, X.F, X.A, s, item, J.qa, J.tcur, J.tnew);
        } else if (K == MK_EMD) {
            m_emd<float>(X.P, X.F, X.A, s, item, J.tnew);
        } else if (K == MK_BT) {
            m_bt<true>(X.P, X.A, s, item, J.tcur, J.tnew, stage, J.dt);
        } else if (K == MK_CELLS) {
            m_cells<true>(X.P, X.F, X.A, s, item, J.qa, J.tcur, J.tnew);
        } else if (K == MK_CHECK) {
            m_check<true>(X.P, X.A, s, item, pos, J.qa, J.tcur, J.tnew, J.flags, J.keys, J.ex, J.flags + 1, J.cap);
        } else {
            m_close<true>(X.P, X.A, s, item, J.qa, J.tnew);
        }
    }
}

// RedistributeGrid of every member that has a list: one CTA per member.
struct RJob {
    int member, qa, tcur, tnew, nwaves;
    const int* list_slot;
    const int* list_cell;
    const int* wave_off;
    int* flags;
};
__global__ void __launch_bounds__(REDIST_THREADS) k_m_redist_batch(const SimStatic* __restrict__ sims,
                                                                   const RJob* __restrict__ jobs) {
    kg_dep_wait();
    const RJob& J = jobs[blockIdx.x];
    const SimStatic& X = sims[J.member];
    m_redist<true>(X.P, X.A, J.list_slot, J.list_cell, J.wave_off, J.nwaves, J.qa, J.tcur, J.tnew, J.flags);
}

}  // namespace kg

namespace {

enum MemberState { ST_FRESH, ST_H1, ST_M, ST_DONE };

struct Member {
    kg_ctx* c = nullptr;
    int next_out = 1;        // the output interval being integrated (kg_run's loop)
    bool finished = false;
    // the step in progress
    int state = ST_DONE;
    bool morpho = false;
    int o[3] = {0, 0, 0}, tnew = 0, guard = 0, ncand = 0;
    double dt = 0.0, cap = 0.0, target = 0.0, dt_m = 0.0;
    std::vector<int> slots;
};

}  // namespace

struct kg_batch {
    cudaStream_t st = nullptr;
    int cap = 0;
    std::vector<Member> mem;            // index = member id
    kg_ctx::Ctl* d_ctl = nullptr;       // contiguous control blocks, one per member slot
    kg_ctx::Ctl* h_ctl = nullptr;       // pinned mirror
    kg::SimStatic* d_static = nullptr;
    std::vector<kg::SimStatic> h_static, up_static;
    // per-launch tables (pinned staging, device copies), sized for `cap` jobs per launch
    static constexpr int NLAUNCH = 8;
    kg::StepArgs* h_args = nullptr;
    kg::StepArgs* d_args = nullptr;
    int* h_idx = nullptr;  // member and prefix arrays: [launch][2][cap + 1]
    int* d_idx = nullptr;
    kg::DtJob* h_dt = nullptr;
    kg::DtJob* d_dt = nullptr;
    kg::ActJob* h_act = nullptr;
    kg::ActJob* d_act = nullptr;
    kg::MJob* h_mjob = nullptr;         // [2][cap]: the M jobs before and after the checks
    kg::MJob* d_mjob = nullptr;
    int* h_mpre = nullptr;              // [2][cap + 1]
    int* d_mpre = nullptr;
    kg::RJob* h_rjob = nullptr;
    kg::RJob* d_rjob = nullptr;
    int grid_m = 0;
    int* d_actout = nullptr;
    int* h_actout = nullptr;
    int actout_cap = 0;
    int grid_hydro = 0, grid_act = 0;
    int launch_no = 0;
    int64_t launches = 0, rounds = 0;
    // CUDA graphs: each device segment of a round (between two waits) is captured from the
    // stream and replayed through one executable graph per segment kind, updated in place
    // (cudaGraphExecUpdate) when the captured segment differs from the last one.
    // A segment's enqueues are first recorded with a byte signature of their parameters
    // (kernel, grid, arguments; copy addresses and sizes): when the signature equals that of
    // the segment kind's executable graph, the graph is launched as it is (the copies read
    // the pinned tables at execution time); otherwise the recorded enqueues are captured
    // and the executable graph updated or instantiated.
    enum { SEG_H = 0, SEG_M1 = 1, SEG_M2 = 2, NSEG = 3 };
    bool use_graphs = true;
    bool capturing = false, recording = false;
    int seg = -1;
    cudaGraphExec_t exec[NSEG] = {nullptr, nullptr, nullptr};
    std::vector<std::function<void()>> ops;
    std::vector<unsigned char> sig_cur, sig[NSEG];
    int64_t graph_launches = 0, graph_updates = 0, graph_instantiations = 0, graph_replays = 0;
    std::string err;
};

namespace {

using namespace kg;

void batch_sync(kg_batch& b) { CK(cudaStreamSynchronize(b.st)); }

// Start a segment of the round (every batched enqueue until seg_end); without graphs the
// enqueues are issued as they come.
void seg_begin(kg_batch& b, int seg) {
    if (!b.use_graphs) return;
    b.recording = true;
    b.seg = seg;
    b.ops.clear();
    b.sig_cur.clear();
}
template <class T>
void sig_add(kg_batch& b, const T& v) {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&v);
    b.sig_cur.insert(b.sig_cur.end(), p, p + sizeof(T));
}
// One batched kernel launch of the round: issued now, or recorded into the segment.
template <typename... KArgs, typename... Args>
void enq_kernel(kg_batch& b, void (*k)(KArgs...), int grid, int block, size_t smem, Args... args) {
    if (!b.recording) {
        CK(kg_launch(k, grid, block, smem, b.st, args...));
        CK(cudaGetLastError());
        return;
    }
    sig_add(b, (const void*)k);
    sig_add(b, grid);
    sig_add(b, block);
    sig_add(b, smem);
    (sig_add(b, args), ...);
    cudaStream_t st = b.st;
    b.ops.push_back([=]() {
        CK(kg_launch(k, grid, block, smem, st, args...));
        CK(cudaGetLastError());
    });
}
// One copy of the round (pinned host tables and device buffers only).
void enq_copy(kg_batch& b, void* dst, const void* src, size_t n, cudaMemcpyKind kind) {
    if (!b.recording) {
        CK(cudaMemcpyAsync(dst, src, n, kind, b.st));
        return;
    }
    sig_add(b, dst);
    sig_add(b, src);
    sig_add(b, n);
    sig_add(b, (int)kind);
    cudaStream_t st = b.st;
    b.ops.push_back([=]() { CK(cudaMemcpyAsync(dst, src, n, kind, st)); });
}
// End the segment and launch it: the segment kind's executable graph as it is when the
// recorded enqueues carry its signature, else the enqueues captured from the stream and the
// executable graph updated in place (or instantiated when its shape changed).
void seg_end(kg_batch& b) {
    if (!b.recording) return;
    b.recording = false;
    cudaGraphExec_t& x = b.exec[b.seg];
    if (x && b.sig_cur == b.sig[b.seg]) {
        CK(cudaGraphLaunch(x, b.st));
        b.graph_launches++;
        b.graph_replays++;
        return;
    }
    CK(cudaStreamBeginCapture(b.st, cudaStreamCaptureModeRelaxed));
    b.capturing = true;
    for (auto& op : b.ops) op();
    cudaGraph_t g = nullptr;
    b.capturing = false;
    CK(cudaStreamEndCapture(b.st, &g));
    if (x) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(x, g, &info) == cudaSuccess) {
            b.graph_updates++;
        } else {
            (void)cudaGetLastError();
            cudaGraphExecDestroy(x);
            x = nullptr;
        }
    }
    cudaError_t e = cudaSuccess;
    if (!x) {
        e = cudaGraphInstantiate(&x, g, 0);
        if (e == cudaSuccess) b.graph_instantiations++;
    }
    cudaGraphDestroy(g);
    CK(e);
    b.sig[b.seg] = b.sig_cur;
    CK(cudaGraphLaunch(x, b.st));
    b.graph_launches++;
}
// Leaves the stream out of capture mode and drops a half-recorded segment when an error
// unwinds through it.
struct SegGuard {
    kg_batch& b;
    ~SegGuard() {
        b.recording = false;
        b.ops.clear();
        if (!b.capturing) return;
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(b.st, &g);
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();
        b.capturing = false;
        if (b.seg >= 0) b.sig[b.seg].clear();
    }
};

// Room for `total` edge-band words (grown before a capture starts: no allocation inside one).
void ensure_actout(kg_batch& b, int total) {
    if (total <= b.actout_cap) return;
    const int cap = std::max(total, 2 * b.actout_cap);  // grows geometrically: few reallocations
    batch_sync(b);
    if (b.d_actout) CK(cudaFree(b.d_actout));
    if (b.h_actout) CK(cudaFreeHost(b.h_actout));
    b.d_actout = nullptr;
    b.h_actout = nullptr;
    b.actout_cap = 0;
    CK(cudaMalloc(&b.d_actout, (size_t)cap * sizeof(int)));
    CK(cudaMallocHost(&b.h_actout, (size_t)cap * sizeof(int)));
    b.actout_cap = cap;
}
int flags_total(kg_batch& b, const std::vector<int>& who) {
    int total = 0;
    for (int id : who) {
        kg_ctx& c = *b.mem[(size_t)id].c;
        total += (int)c.active.size() * ((c.SC + 255) / 256);
    }
    return total;
}

// Rebuild the member table on the host and upload it when it changed.
void refresh_static(kg_batch& b) {
    b.h_static.assign((size_t)b.cap, SimStatic{});
    for (int i = 0; i < b.cap; ++i) {
        const Member& m = b.mem[(size_t)i];
        if (!m.c) continue;
        const kg_ctx& c = *m.c;
        SimStatic& X = b.h_static[(size_t)i];
        X.A = c.A;
        X.P = c.dp;
        X.F = params32(c.dp);
        X.src = c.d_src;
        X.blocks = c.d_blocks;
        X.slots = c.d_active;
        X.nblocks = (int)c.blocks.size();
        X.nactive = (int)c.active.size();
    }
    if (b.up_static.size() == b.h_static.size() &&
        std::memcmp(b.up_static.data(), b.h_static.data(), b.h_static.size() * sizeof(SimStatic)) == 0)
        return;
    CK(cudaMemcpyAsync(b.d_static, b.h_static.data(), b.h_static.size() * sizeof(SimStatic), cudaMemcpyHostToDevice, b.st));
    batch_sync(b);  // the host table is the copy's source
    b.up_static = b.h_static;
}

// One batched hydraulic pass over the listed (member, args) jobs.
void launch_hydro_batch(kg_batch& b, const std::vector<int>& who, const std::vector<StepArgs>& args) {
    int n = (int)who.size();
    if (n == 0) return;
    int L = b.launch_no++ % kg_batch::NLAUNCH;
    StepArgs* ha = b.h_args + (size_t)L * b.cap;
    int* hm = b.h_idx + (size_t)L * 2 * (b.cap + 1);
    int* hp = hm + (b.cap + 1);
    int total = 0;
    for (int k = 0; k < n; ++k) {
        ha[k] = args[(size_t)k];
        hm[k] = who[(size_t)k];
        hp[k] = total;
        total += (int)b.mem[(size_t)who[(size_t)k]].c->blocks.size();
    }
    StepArgs* da = b.d_args + (size_t)L * b.cap;
    int* dm = b.d_idx + (size_t)L * 2 * (b.cap + 1);
    int* dp = dm + (b.cap + 1);
    enq_copy(b, da, ha, (size_t)n * sizeof(StepArgs), cudaMemcpyHostToDevice);
    enq_copy(b, dm, hm, (size_t)2 * (b.cap + 1) * sizeof(int), cudaMemcpyHostToDevice);
    if (total == 0) return;
    int grid = std::min(total, b.grid_hydro);
    enq_kernel(b, k_hydro32_batch, grid, NT, sizeof(Hydro32Smem), (const SimStatic*)b.d_static, (const StepArgs*)da,
               (const int*)dm, (const int*)dp, n, total);
    b.launches++;
}

// The pass arguments a member's single-simulation path would launch with (launch_pass).
StepArgs member_args(kg_ctx& c, StepArgs S, int word) {
    S.cfl_min = c.d_cfl + word;
    S.partial = partial(c);
    return S;
}

// Queue the three RK stages for the listed members (the batched queue_hydraulic): fresh
// members read their dt on the device, the others use the host dt; `m_gates` adds the
// M-phase gates (refine flag and RHS check).
void queue_stages_batch(kg_batch& b, const std::vector<int>& who, bool m_gates) {
    std::vector<StepArgs> a1, a2, a3;
    for (int id : who) {
        Member& m = b.mem[(size_t)id];
        kg_ctx& c = *m.c;
        bool fresh = m.state == ST_FRESH;
        int q_in = m_gates ? m.o[0] : c.qcur, e_set = m_gates ? 1 : 0, topo = m_gates ? m.tnew : c.tcur;
        int q_s1 = m_gates ? m.o[1] : m.o[0], q_s2 = m_gates ? m.o[2] : m.o[1], q_out = m_gates ? m.o[1] : m.o[0];
        double dt = fresh ? 0.0 : m.dt;
        double nextT = c.t + dt;
        StepArgs S{};
        S.q_in = q_in; S.q_s1 = q_s1; S.q_s2 = q_s2; S.q_out = q_out; S.e_set = e_set; S.topo = topo;
        S.q_tc = c.qcur; S.topo_tc = c.tcur;
        // The running maxima change only in the first accepted half-step of a step (they read
        // the step-start state with strict comparisons); later half-steps skip them.
        if (fresh) c.maxima_done = false;
        S.dt = dt; S.dtp = fresh ? c.d_dt : nullptr; S.t_grid = c.t; S.do_maxima = (m_gates || c.maxima_done) ? 0 : 1;
        int g0 = 0;
        if (m_gates) {
            S.gate_flag = c.d_mflags;
            S.gate[0] = c.d_cfl + W_RHS;
            S.gate_s1[0] = 1;
            g0 = 1;
        }
        if (!fresh) c.dt = dt;
        S.mode = MODE_S1; S.t_rhs = nextT; S.tmode = 1; S.ngate = g0;
        a1.push_back(member_args(c, S, W_S1));
        S.mode = MODE_S2; S.t_rhs = c.t + 0.5 * dt; S.tmode = 2;
        S.gate[g0] = c.d_cfl + W_S1; S.gate_s1[g0] = 0; S.ngate = g0 + 1;
        a2.push_back(member_args(c, S, W_S2));
        S.mode = MODE_S3; S.t_rhs = nextT; S.t_max = nextT; S.tmode = 1;
        S.gate[g0 + 1] = c.d_cfl + W_S2; S.gate_s1[g0 + 1] = 0; S.ngate = g0 + 2;
        a3.push_back(member_args(c, S, W_S3));
    }
    launch_hydro_batch(b, who, a1);
    launch_hydro_batch(b, who, a2);
    launch_hydro_batch(b, who, a3);
}

// Edge-band flags of the listed members' results (q_out, topo) into the batch buffer;
// offsets[k] is where member who[k]'s words start.
void queue_flags_batch(kg_batch& b, const std::vector<int>& who, const std::vector<int>& q, const std::vector<int>& topo,
                       std::vector<int>& offsets) {
    int n = (int)who.size();
    offsets.assign((size_t)n, 0);
    if (n == 0) return;
    int* hp = b.h_idx + (size_t)(kg_batch::NLAUNCH) * 2 * (b.cap + 1);  // the flags job prefix
    int total = 0;
    for (int k = 0; k < n; ++k) {
        kg_ctx& c = *b.mem[(size_t)who[(size_t)k]].c;
        int per = (c.SC + 255) / 256;
        b.h_act[k] = ActJob{who[(size_t)k], q[(size_t)k], topo[(size_t)k], per};
        hp[k] = total;
        offsets[(size_t)k] = total;
        total += (int)c.active.size() * per;
    }
    if (total > b.actout_cap) throw KgError(KG_ERR_STATE, "edge-band buffer not sized before the segment");
    int* dp = b.d_idx + (size_t)(kg_batch::NLAUNCH) * 2 * (b.cap + 1);
    enq_copy(b, b.d_act, b.h_act, (size_t)n * sizeof(ActJob), cudaMemcpyHostToDevice);
    enq_copy(b, dp, hp, (size_t)n * sizeof(int), cudaMemcpyHostToDevice);
    if (total == 0) return;
    enq_kernel(b, k_act_flags_batch, std::min(total, b.grid_act), 256, 0, (const SimStatic*)b.d_static, (const ActJob*)b.d_act,
               (const int*)dp, n, total, b.d_actout);
    b.launches++;
    enq_copy(b, b.h_actout, b.d_actout, (size_t)total * sizeof(int), cudaMemcpyDeviceToHost);
}

// Reset every member's CFL words (one copy; the other control words are left to the
// kernels that own them).
void reset_ctl(kg_batch& b) {
    for (int i = 0; i < b.cap; ++i)
        for (int k = 0; k < 4; ++k) b.h_ctl[i].cfl[k] = HUGE_BITS;
    enq_copy(b, b.d_ctl, b.h_ctl, (size_t)b.cap * sizeof(kg_ctx::Ctl), cudaMemcpyHostToDevice);
}
void read_ctl(kg_batch& b) {
    enq_copy(b, b.h_ctl, b.d_ctl, (size_t)b.cap * sizeof(kg_ctx::Ctl), cudaMemcpyDeviceToHost);
}
// The end of a segment: the control words come back, the segment runs, one wait.
void collect_ctl(kg_batch& b) {
    read_ctl(b);
    seg_end(b);
    batch_sync(b);
}

// The end of an accepted step (the tail of integrate_step).
void finish_step(Member& m, int newcur) {
    kg_ctx& c = *m.c;
    c.qcur = newcur;
    if (m.morpho) c.tcur = m.tnew;
    c.t = m.morpho ? c.t0 + 2.0 * m.dt : c.t0 + m.dt;
    c.dt = m.dt;
    c.steps++;
    c.cell_updates += (int64_t)c.active.size() * c.SC * (m.morpho ? 2 : 1);
    c.src_override = false;
    m.state = ST_DONE;
    if (c.t >= m.target) {
        m.next_out++;
        int Nout = c.p.Nout > 0 ? c.p.Nout : 100;
        if (m.next_out > Nout) m.finished = true;
    }
}

// A refused attempt: back to the first H with the refined dt (the loop of integrate_step).
void refuse(Member& m) {
    m.c->rejected++;
    m.c->dt = m.dt;
    m.state = ST_H1;
}

// Guard of each attempt (integrate_step's loop head).
void guard(Member& m) {
    if (++m.guard > 100000 || !(m.dt > 0.0)) throw KgError(KG_ERR_DT, "time step collapsed");
}

// Phase H: RHS + device dt for fresh members, the three stages for fresh and retrying
// members, flags for hydraulic-only members; one wait; the host's tests.
void phase_h(kg_batch& b, const std::vector<int>& who) {
    std::vector<int> fresh;
    std::vector<StepArgs> ra;
    for (int id : who) {
        Member& m = b.mem[(size_t)id];
        kg_ctx& c = *m.c;
        if (c.prec == KG_PREC_FP32 && c.tdirty[c.tcur]) {
            bind_constants(c);
            refresh_topo32(c, c.tcur);
        }
        if (m.state == ST_FRESH) {
            fresh.push_back(id);
            ra.push_back(member_args(c, rhs_args(c, c.qcur, 0, c.tcur, c.t), W_RHS));
        }
    }
    std::vector<int> hydro_only;
    for (int id : who)
        if (!b.mem[(size_t)id].morpho) hydro_only.push_back(id);
    ensure_actout(b, flags_total(b, hydro_only));
    SegGuard seg_guard{b};
    seg_begin(b, kg_batch::SEG_H);
    reset_ctl(b);
    launch_hydro_batch(b, fresh, ra);
    if (!fresh.empty()) {
        int n = (int)fresh.size();
        for (int k = 0; k < n; ++k) {
            Member& m = b.mem[(size_t)fresh[(size_t)k]];
            b.h_dt[k] = DtJob{m.c->d_cfl + W_RHS, m.c->d_dt, m.cap, partial(*m.c), fresh[(size_t)k]};
        }
        enq_copy(b, b.d_dt, b.h_dt, (size_t)n * sizeof(DtJob), cudaMemcpyHostToDevice);
        enq_kernel(b, k_dt_batch, (n + 127) / 128, 128, 0, (const SimStatic*)b.d_static, (const DtJob*)b.d_dt, n);
        b.launches++;
    }
    queue_stages_batch(b, who, false);
    std::vector<int> fw, fq, ft, off;
    for (int id : who)
        if (!b.mem[(size_t)id].morpho) {
            fw.push_back(id);
            fq.push_back(b.mem[(size_t)id].o[0]);
            ft.push_back(b.mem[(size_t)id].c->tcur);
        }
    queue_flags_batch(b, fw, fq, ft, off);
    collect_ctl(b);
    size_t fk = 0;
    for (int id : who) {
        Member& m = b.mem[(size_t)id];
        kg_ctx& c = *m.c;
        if (m.state == ST_FRESH) {
            double adv = mn(advised(c, c.h_cfl[W_RHS], 1), m.cap);
            double ddt = c.h_ctl->dt;
            if (!(adv == ddt) && !(adv != adv && ddt != ddt)) throw KgError(KG_ERR_CUDA, "device-side dt differs from the host's");
            c.dt = adv;
            m.dt = adv;
        }
        guard(m);
        const int* chunks = nullptr;
        if (!m.morpho) {
            while (fk < fw.size() && fw[fk] != id) ++fk;
            chunks = b.h_actout + off[fk];
        }
        bool rej = finish_hydraulic(c, m.dt, m.o[0], c.tcur, !m.morpho, chunks);
        if (rej) { refuse(m); continue; }
        c.maxima_done = true;
        if (!m.morpho) finish_step(m, m.o[0]);
        else m.state = ST_M;
    }
}

// Upload M job table t (0: the operator and its checks, 1: after the checks).
int upload_mjobs(kg_batch& b, int t, const std::vector<int>& who) {
    MJob* hj = b.h_mjob + (size_t)t * b.cap;
    int* hp = b.h_mpre + (size_t)t * (b.cap + 1);
    int total = 0;
    for (size_t k = 0; k < who.size(); ++k) {
        Member& m = b.mem[(size_t)who[k]];
        kg_ctx& c = *m.c;
        int per = (c.SV + 255) / 256;
        hj[k] = MJob{who[k], per, m.o[0], c.tcur, m.tnew, c.cand_cap, m.dt_m, c.d_mflags, c.d_ckey, c.d_cex};
        hp[k] = total;
        total += (int)c.active.size() * per;
    }
    enq_copy(b, b.d_mjob + (size_t)t * b.cap, hj, who.size() * sizeof(MJob), cudaMemcpyHostToDevice);
    enq_copy(b, b.d_mpre + (size_t)t * (b.cap + 1), hp, who.size() * sizeof(int), cudaMemcpyHostToDevice);
    return total;
}
template <int K>
void launch_m(kg_batch& b, int t, int n, int total, int stage = 0) {
    if (n == 0 || total == 0) return;
    enq_kernel(b, k_m_batch<K>, std::min(total, b.grid_m), 256, 0, (const SimStatic*)b.d_static,
               (const MJob*)(b.d_mjob + (size_t)t * b.cap), (const int*)(b.d_mpre + (size_t)t * (b.cap + 1)), n, total,
               stage);
    b.launches++;
}

// Phase M: the morphodynamic operator of every listed member (one launch per step kind
// for all of them), its checks and redistribution, then the batched RHS check and second
// H.
void phase_m(kg_batch& b, const std::vector<int>& who) {
    for (int id : who) {
        Member& m = b.mem[(size_t)id];
        kg_ctx& c = *m.c;
        m.dt_m = 2.0 * m.dt;
        m.slots.clear();
        for (int t : c.active) m.slots.push_back(T(c, t).slot);
        int need = (int)m.slots.size() * c.SC;
        if (need > c.cand_cap) {
            cudaFree(c.d_ckey); cudaFree(c.d_cex); cudaFree(c.d_rslot); cudaFree(c.d_rcell); cudaFree(c.d_rwave);
            c.cand_cap = std::max(need, 2 * c.cand_cap);
            CK(cudaMalloc(&c.d_ckey, (size_t)c.cand_cap * sizeof(unsigned long long)));
            CK(cudaMalloc(&c.d_cex, (size_t)c.cand_cap * sizeof(double)));
            CK(cudaMalloc(&c.d_rslot, (size_t)c.cand_cap * sizeof(int)));
            CK(cudaMalloc(&c.d_rcell, (size_t)c.cand_cap * sizeof(int)));
            CK(cudaMalloc(&c.d_rwave, ((size_t)c.cand_cap + 1) * sizeof(int)));
        }
        c.launches += 11;
    }
    SegGuard seg_guard{b};
    seg_begin(b, kg_batch::SEG_M1);
    reset_ctl(b);
    int n = (int)who.size();
    int total = upload_mjobs(b, 0, who);
    launch_m<MK_INIT>(b, 0, n, total);
    for (int stage = 1; stage <= 3; ++stage) {
        launch_m<MK_EMD>(b, 0, n, total);
        launch_m<MK_BT>(b, 0, n, total, stage);
        launch_m<MK_CELLS>(b, 0, n, total);
    }
    launch_m<MK_CHECK>(b, 0, n, total);
    collect_ctl(b);
    std::vector<int> go, listed;
    for (int id : who) {
        Member& m = b.mem[(size_t)id];
        kg_ctx& c = *m.c;
        if (c.h_ctl->mflag != 0) {
            m.dt_m = 0.5 * m.dt_m;
            m.dt = 0.5 * m.dt_m;
            refuse(m);
            continue;
        }
        m.ncand = c.h_ctl->ncand;
        go.push_back(id);
        if (m.ncand > 0) listed.push_back(id);
    }
    // Redistribution lists of the members that have one (one wait for all read-backs).
    std::vector<std::vector<unsigned long long>> keys(listed.size());
    std::vector<std::vector<double>> exs(listed.size());
    for (size_t k = 0; k < listed.size(); ++k) {
        Member& m = b.mem[(size_t)listed[k]];
        kg_ctx& c = *m.c;
        keys[k].resize((size_t)m.ncand);
        exs[k].resize((size_t)m.ncand);
        CK(cudaMemcpyAsync(keys[k].data(), c.d_ckey, (size_t)m.ncand * sizeof(unsigned long long), cudaMemcpyDeviceToHost, b.st));
        CK(cudaMemcpyAsync(exs[k].data(), c.d_cex, (size_t)m.ncand * sizeof(double), cudaMemcpyDeviceToHost, b.st));
    }
    if (!listed.empty()) batch_sync(b);
    for (size_t k = 0; k < listed.size(); ++k) {
        Member& m = b.mem[(size_t)listed[k]];
        kg_ctx& c = *m.c;
        const auto& key = keys[k];
        const auto& ex = exs[k];
        int ncand = m.ncand;
        std::vector<int> ord((size_t)ncand);
        for (int q = 0; q < ncand; ++q) ord[(size_t)q] = q;
        std::sort(ord.begin(), ord.end(), [&](int x, int y) {
            if (ex[(size_t)x] != ex[(size_t)y]) return ex[(size_t)x] < ex[(size_t)y];
            return key[(size_t)x] < key[(size_t)y];
        });
        std::vector<int> ls, lc, woff;
        redistribution_waves(c, m.slots, key, ord, ls, lc, woff);
        int nw = (int)woff.size() - 1;
        c.redist_cells += ncand;
        c.redist_waves += nw;
        c.redist_walks++;
        CK(cudaMemcpyAsync(c.d_rslot, ls.data(), (size_t)ncand * sizeof(int), cudaMemcpyHostToDevice, c.st));
        CK(cudaMemcpyAsync(c.d_rcell, lc.data(), (size_t)ncand * sizeof(int), cudaMemcpyHostToDevice, c.st));
        CK(cudaMemcpyAsync(c.d_rwave, woff.data(), woff.size() * sizeof(int), cudaMemcpyHostToDevice, c.st));
        b.h_rjob[k] = RJob{listed[k], m.o[0], c.tcur, m.tnew, nw, c.d_rslot, c.d_rcell, c.d_rwave, c.d_mflags};
        c.launches++;
    }
    if (!listed.empty()) {
        CK(cudaMemcpyAsync(b.d_rjob, b.h_rjob, listed.size() * sizeof(RJob), cudaMemcpyHostToDevice, b.st));
        CK(kg_launch(k_m_redist_batch, (int)listed.size(), REDIST_THREADS, 0, b.st, b.d_static, b.d_rjob));
        CK(cudaGetLastError());
        b.launches++;
    }
    if (go.empty()) return;
    // Interfacial topography of the new bed and the M result, for every member at once.
    std::vector<int> whole;
    for (int id : go) {
        Member& m = b.mem[(size_t)id];
        kg_ctx& c = *m.c;
        c.launches += 1;
        if (c.tdirty[m.tnew] > 1) whole.push_back(id);
    }
    ensure_actout(b, flags_total(b, go));
    // A member whose ghost tiles never had the factors of this topography set rebuilds them
    // through context-owned lists (host copies), so that segment is not captured.
    if (whole.empty()) seg_begin(b, kg_batch::SEG_M2);
    int ng = (int)go.size();
    int tg = upload_mjobs(b, 1, go);
    // interfacial topography, the M result and the active tiles' factor cache, fused
    launch_m<MK_CLOSE>(b, 1, ng, tg);
    for (int id : whole) {            // ghost factors too where they were never built
        kg_ctx& c = *b.mem[(size_t)id].c;
        bind_constants(c);
        refresh_topo32(c, b.mem[(size_t)id].tnew);
    }
    std::vector<StepArgs> ra;
    for (int id : go) {
        Member& m = b.mem[(size_t)id];
        kg_ctx& c = *m.c;
        c.tdirty[m.tnew] = 0;
        c.t = c.t0 + m.dt;
        c.dt = m.dt;
        ra.push_back(member_args(c, rhs_args(c, m.o[0], 1, m.tnew, c.t), W_RHS));
    }
    launch_hydro_batch(b, go, ra);
    queue_stages_batch(b, go, true);
    std::vector<int> fq, ft, off;
    for (int id : go) {
        fq.push_back(b.mem[(size_t)id].o[1]);
        ft.push_back(b.mem[(size_t)id].tnew);
    }
    queue_flags_batch(b, go, fq, ft, off);
    collect_ctl(b);
    for (size_t k = 0; k < go.size(); ++k) {
        Member& m = b.mem[(size_t)go[k]];
        kg_ctx& c = *m.c;
        if (c.h_ctl->mflag != 0) {
            c.t = c.t0;
            m.dt_m = 0.5 * m.dt_m;
            m.dt = 0.5 * m.dt_m;
            refuse(m);
            continue;
        }
        double adv = advised(c, c.h_cfl[W_RHS], 1);
        if (adv < m.dt) {
            if ((m.dt - adv) / m.dt < 0.1) m.dt = 0.9 * m.dt;
            else m.dt = adv;
            c.t = c.t0;
            refuse(m);
            continue;
        }
        if (!finish_hydraulic(c, m.dt, m.o[1], m.tnew, true, b.h_actout + off[k])) {
            finish_step(m, m.o[1]);
            continue;
        }
        c.t = c.t0;
        refuse(m);
    }
}

// Prepare one step of a member (the head of integrate_step).
void prepare(kg_batch& b, Member& m) {
    kg_ctx& c = *m.c;
    bind_constants(c);
    if (!c.sources_loaded) throw KgError(KG_ERR_STATE, "kg_load_sources must be called before stepping");
    m.target = c.p.tstart + m.next_out * c.DeltaT;
    check_near_boundaries(c);
    rebuild_blocks(c);
    m.morpho = c.p.MorphodynamicsOn != 0;
    int k = 0;
    for (int q = 0; q < 4; ++q)
        if (q != c.qcur) m.o[k++] = q;
    m.tnew = 1 - c.tcur;
    double tmax = mn(m.target, next_flux_time(c, c.t));
    m.cap = m.morpho ? 0.5 * (tmax - c.t) : tmax - c.t;
    c.t0 = c.t;
    m.guard = 0;
    m.state = ST_FRESH;
    (void)b;
}

// One round: every live member advances its own step by one phase.  A member whose
// previous step is complete starts the next one (prepare), members at the first H (fresh
// or retrying) share the batched H phase, and members whose first H was accepted share
// the M phase; a member that completes its step starts the next one in the next round,
// so no member waits for another's retries.
void batch_step(kg_batch& b) {
    // A round makes at most NLAUNCH (8) batched hydraulic launches: the RHS and three stages
    // of H, the RHS check and three stages of the second H.  Numbering them from 0 every round
    // gives each position the same table slot, so a segment captured in one round has the
    // same kernel arguments as the last one whenever its jobs are unchanged.
    b.launch_no = 0;
    std::vector<int> live;
    for (int i = 0; i < b.cap; ++i)
        if (b.mem[(size_t)i].c && !b.mem[(size_t)i].finished) live.push_back(i);
    for (int id : live) {
        Member& m = b.mem[(size_t)id];
        if (m.state != ST_DONE) continue;
        // kg_integrate_to skips an interval that is already reached
        int Nout = m.c->p.Nout > 0 ? m.c->p.Nout : 100;
        while (!m.finished && m.c->t >= m.c->p.tstart + m.next_out * m.c->DeltaT) {
            m.next_out++;
            if (m.next_out > Nout) m.finished = true;
        }
        if (!m.finished) prepare(b, m);
    }
    refresh_static(b);
    std::vector<int> h, mm;
    for (int id : live) {
        int s = b.mem[(size_t)id].state;
        if (!b.mem[(size_t)id].finished && (s == ST_FRESH || s == ST_H1)) h.push_back(id);
    }
    if (!h.empty()) phase_h(b, h);
    for (int id : live)
        if (b.mem[(size_t)id].state == ST_M) mm.push_back(id);
    if (!mm.empty()) phase_m(b, mm);
    b.rounds++;
}

}  // namespace

extern "C" {

void kg_batch_destroy(kg_batch* b);

int kg_batch_create(int32_t max_members, kg_batch** out) {
    if (!out || max_members < 1) return KG_ERR_PARAM;
    *out = nullptr;
    std::lock_guard<std::recursive_mutex> lock(g_api_mu);
    kg_batch* b = new kg_batch();
    try {
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) throw KgError(KG_ERR_CUDA, "no CUDA device is available");
        b->cap = max_members;
        b->mem.resize((size_t)max_members);
        CK(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
        CK(cudaMalloc(&b->d_ctl, (size_t)max_members * sizeof(kg_ctx::Ctl)));
        CK(cudaMemset(b->d_ctl, 0, (size_t)max_members * sizeof(kg_ctx::Ctl)));
        CK(cudaMallocHost(&b->h_ctl, (size_t)max_members * sizeof(kg_ctx::Ctl)));
        CK(cudaMalloc(&b->d_static, (size_t)max_members * sizeof(SimStatic)));
        CK(cudaMallocHost(&b->h_args, (size_t)kg_batch::NLAUNCH * max_members * sizeof(StepArgs)));
        CK(cudaMalloc(&b->d_args, (size_t)kg_batch::NLAUNCH * max_members * sizeof(StepArgs)));
        size_t nidx = (size_t)(kg_batch::NLAUNCH + 1) * 2 * (max_members + 1);
        CK(cudaMallocHost(&b->h_idx, nidx * sizeof(int)));
        CK(cudaMalloc(&b->d_idx, nidx * sizeof(int)));
        CK(cudaMallocHost(&b->h_dt, (size_t)max_members * sizeof(DtJob)));
        CK(cudaMalloc(&b->d_dt, (size_t)max_members * sizeof(DtJob)));
        CK(cudaMallocHost(&b->h_act, (size_t)max_members * sizeof(ActJob)));
        CK(cudaMalloc(&b->d_act, (size_t)max_members * sizeof(ActJob)));
        CK(cudaMallocHost(&b->h_mjob, (size_t)2 * max_members * sizeof(MJob)));
        CK(cudaMalloc(&b->d_mjob, (size_t)2 * max_members * sizeof(MJob)));
        CK(cudaMallocHost(&b->h_mpre, (size_t)2 * (max_members + 1) * sizeof(int)));
        CK(cudaMalloc(&b->d_mpre, (size_t)2 * (max_members + 1) * sizeof(int)));
        CK(cudaMallocHost(&b->h_rjob, (size_t)max_members * sizeof(RJob)));
        CK(cudaMalloc(&b->d_rjob, (size_t)max_members * sizeof(RJob)));
        CK(cudaFuncSetAttribute(k_hydro32_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Hydro32Smem)));
        int dev = 0, sms = 0, occ = 0, occa = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_hydro32_batch, NT, sizeof(Hydro32Smem)));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occa, k_act_flags_batch, 256, 0));
        b->grid_hydro = sms * std::max(occ, 1);
        int occm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occm, k_m_batch<MK_CELLS>, 256, 0));
        b->grid_m = sms * std::max(occm, 1);
        b->grid_act = sms * std::max(occa, 1);
    } catch (const KgError& e) {
        int code = e.code;
        kg_batch_destroy(b);
        return code;
    }
    *out = b;
    return KG_OK;
}

const char* kg_batch_last_error(const kg_batch* b) { return b ? b->err.c_str() : "null batch"; }

int kg_batch_add(kg_batch* b, const kg_params* params, const double* b0, int64_t nx1, int64_t ny1, int32_t* id) {
    if (!b || !params || !id) return KG_ERR_PARAM;
    std::lock_guard<std::recursive_mutex> lock(g_api_mu);
    int slot = -1;
    for (int i = 0; i < b->cap; ++i)
        if (!b->mem[(size_t)i].c) { slot = i; break; }
    if (slot < 0) { b->err = "the batch is full"; return KG_ERR_STATE; }
    kg_ctx* c = nullptr;
    int rc = kg_create(params, KG_PREC_FP32, &c);
    if (rc != KG_OK) { b->err = "kg_create failed: " + g_create_err; return rc; }
    try {
        // the member runs on the batch stream and keeps its control words in the batch
        CK(cudaStreamSynchronize(c->st));
        CK(cudaStreamDestroy(c->st));
        c->st = b->st;
        c->own_stream = false;
        CK(cudaFree(c->d_ctl));
        CK(cudaFreeHost(c->h_ctl));
        c->own_ctl = false;
        c->d_ctl = b->d_ctl + slot;
        c->h_ctl = b->h_ctl + slot;
        c->d_cfl = c->d_ctl->cfl;
        c->d_dt = &c->d_ctl->dt;
        c->d_mflags = &c->d_ctl->mflag;
        c->d_ncand = &c->d_ctl->ncand;
        c->h_cfl = c->h_ctl->cfl;
        g_const_owner = nullptr;
        if (b0) {
            rc = kg_upload_b0(c, b0, nx1, ny1);
            if (rc != KG_OK) throw KgError(rc, c->err);
        }
        rc = kg_load_sources(c);
        if (rc != KG_OK) throw KgError(rc, c->err);
    } catch (const KgError& e) {
        b->err = e.what();
        kg_destroy(c);
        return e.code;
    }
    b->mem[(size_t)slot] = Member{};
    b->mem[(size_t)slot].c = c;
    *id = slot;
    return KG_OK;
}

kg_ctx* kg_batch_member(kg_batch* b, int32_t id) {
    if (!b || id < 0 || id >= b->cap) return nullptr;
    return b->mem[(size_t)id].c;
}

int kg_batch_remove(kg_batch* b, int32_t id) {
    if (!b || id < 0 || id >= b->cap || !b->mem[(size_t)id].c) return KG_ERR_PARAM;
    std::lock_guard<std::recursive_mutex> lock(g_api_mu);
    cudaStreamSynchronize(b->st);
    kg_destroy(b->mem[(size_t)id].c);
    b->mem[(size_t)id] = Member{};
    return KG_OK;
}

int kg_batch_step(kg_batch* b, int32_t* live) {
    if (!b) return KG_ERR_PARAM;
    std::lock_guard<std::recursive_mutex> lock(g_api_mu);
    try {
        batch_step(*b);
    } catch (const KgError& e) {
        b->err = e.what();
        return e.code;
    }
    if (live) {
        int n = 0;
        for (int i = 0; i < b->cap; ++i)
            if (b->mem[(size_t)i].c && !b->mem[(size_t)i].finished) ++n;
        *live = n;
    }
    return KG_OK;
}

int kg_batch_finished(kg_batch* b, int32_t id, int32_t* finished) {
    if (!b || !finished || id < 0 || id >= b->cap || !b->mem[(size_t)id].c) return KG_ERR_PARAM;
    Member& m = b->mem[(size_t)id];
    int Nout = m.c->p.Nout > 0 ? m.c->p.Nout : 100;
    while (!m.finished && m.c->t >= m.c->p.tstart + m.next_out * m.c->DeltaT) {
        m.next_out++;
        if (m.next_out > Nout) m.finished = true;
    }
    *finished = m.finished ? 1 : 0;
    return KG_OK;
}

int kg_batch_stats(kg_batch* b, int64_t* launches, int64_t* rounds) {
    if (!b || !launches || !rounds) return KG_ERR_PARAM;
    *launches = b->launches;
    *rounds = b->rounds;
    return KG_OK;
}

void* kg_batch_stream(kg_batch* b) { return b ? (void*)b->st : nullptr; }

int kg_batch_set_graphs(kg_batch* b, int32_t enable) {
    if (!b) return KG_ERR_PARAM;
    std::lock_guard<std::recursive_mutex> lock(g_api_mu);
    b->use_graphs = enable != 0;
    return KG_OK;
}

int kg_batch_graph_stats(kg_batch* b, int64_t out[4]) {
    if (!b || !out) return KG_ERR_PARAM;
    out[0] = b->graph_launches;
    out[1] = b->graph_updates;
    out[2] = b->graph_instantiations;
    out[3] = b->graph_replays;
    return KG_OK;
}

void kg_batch_destroy(kg_batch* b) {
    if (!b) return;
    std::lock_guard<std::recursive_mutex> lock(g_api_mu);
    if (b->st) cudaStreamSynchronize(b->st);
    for (cudaGraphExec_t& x : b->exec)
        if (x) cudaGraphExecDestroy(x);
    for (Member& m : b->mem)
        if (m.c) kg_destroy(m.c);
    cudaFree(b->d_ctl);
    cudaFree(b->d_static);
    cudaFree(b->d_args);
    cudaFree(b->d_idx);
    cudaFree(b->d_dt);
    cudaFree(b->d_act);
    cudaFree(b->d_mjob);
    cudaFree(b->d_mpre);
    cudaFree(b->d_rjob);
    if (b->h_mjob) cudaFreeHost(b->h_mjob);
    if (b->h_mpre) cudaFreeHost(b->h_mpre);
    if (b->h_rjob) cudaFreeHost(b->h_rjob);
    cudaFree(b->d_actout);
    if (b->h_ctl) cudaFreeHost(b->h_ctl);
    if (b->h_args) cudaFreeHost(b->h_args);
    if (b->h_idx) cudaFreeHost(b->h_idx);
    if (b->h_dt) cudaFreeHost(b->h_dt);
    if (b->h_act) cudaFreeHost(b->h_act);
    if (b->h_actout) cudaFreeHost(b->h_actout);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
}

}  // extern "C"
