// engine.cu -- host side of libmdgb: the C ABI declared in include/mdgb.h.
//
// Drives the kernels of kernels_step.cu / kernels_list.cu / kernels_force.cu
// on one CUDA stream per handle.  One integrator step (integrator.rs:14-59)
// is three or four launches:
//   k_pre        (cooperative)  coupling reductions -> kick/drift/wrap -> rebuild
//                               check -> [cell sort, only if needed]
//   k_build_list                Verlet list of the rebuilt replicas (else returns)
//   k_force_*                   LJ forces + second half kick (+ on NVE chunks the
//                               next step's kick and drift, double-buffered)
//   k_force_band (mixed path)   the atoms with a pair in the FP32-undecidable
//                               band around r_cut, with FP64 decisions
// Steps run in chunks; before each chunk the engine snapshots the mutable
// device state, and if the chunk reports a neighbour-list overflow it grows
// the list, restores the snapshot and re-runs the chunk -- so capacity
// misses never surface as wrong results.  Chunks can be captured once into a
// CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mdgb.h"
#include "host_math.h"
#include "mdgb_internal.cuh"

namespace mdgb {
__global__ void k_pre(Dev d, StepParams sp);
__global__ void k_macro(Dev d, StepParams sp, int sel);
__global__ void k_apply_pending(Dev d);
__global__ void k_apply_pending_box(Dev d);
__global__ void k_gather_out(Dev d, double*, double*, double*, double*, double*);
__global__ void k_scatter_in(Dev d, const double*, const double*, const int*, const int*);
__global__ void k_scatter_forces(Dev d, const double*, const double*, const double*);
__global__ void k_pairs(Dev d, long long capacity, int* out_i, int* out_j, unsigned long long* count);
using force_fn = void (*)(Dev, StepParams);
force_fn force_kernel(int tpa, int precision, bool single, bool kick, bool persistent, bool noe);
using band_fn = void (*)(Dev, StepParams, int);
band_fn band_kernel(int precision);
}  // namespace mdgb

using namespace mdgb;

namespace {

struct LJ {
    double sigma = 0.3418, eps = 1.712, rc = 0.0, ucut = 0.0;  // potential.rs:96 default
    bool set = false;
};

void lj_finish(LJ& p) {
    double out[4];
    mdgb_lj_new(p.sigma, p.eps, out);
    p.rc = out[2];
    p.ucut = out[3];
}

struct ProfEvent { cudaEvent_t a, b; int kind; };

}  // namespace

struct mdgb_engine {
    mdgb_config cfg{};
    std::string err;
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    int pre_blocks_per_sm = 0;
    int force_blocks_per_sm[4] = {0, 0, 0, 0};
    LJ pot[MAX_TYPES][MAX_TYPES];
    LJ pot_default;

    // state
    bool has_state = false;
    bool forces_valid = false;
    int ntot = 0, nrep = 0, ntypes = 0, ntiles = 0, ncells = 0;
    std::vector<int64_t> offsets;
    std::vector<double> mass;
    std::vector<RepDev> rep_host;
    double rlist = 0, rcmax = 0, skin = 0;
    int cap = 0;
    int tpa = 1;                     // default / single-class threads per atom
    bool tuned = false;
    // size classes of replicas (by atom count): their tiles, threads per atom
    static constexpr int NCLASS = 3;
    std::vector<int> class_of;       // per replica
    int class_tpa[NCLASS] = {1, 1, 1};
    int class_ntiles[NCLASS] = {0, 0, 0};
    int class_tile_off[NCLASS] = {0, 0, 0};   // offset into dev.tile_order
    int class_nrep[NCLASS] = {0, 0, 0};

    Dev dev{};
    // allocations
    std::vector<void*> allocs;
    void* nbr_alloc = nullptr;
    // snapshot buffers (chunk retry)
    double4_32a* snap_pos = nullptr;
    double* snap_d = nullptr;   // [8][N]
    int* snap_i = nullptr;      // [4][N]: orig, rank, cell, slot_of_rank
    float4* snap_mir0 = nullptr;
    RepDev* snap_rep = nullptr;
    // staging
    double* d_out = nullptr;     // [11][N] gather-out staging
    double* h_pin = nullptr;     // pinned host staging [11][N]
    int* d_in_i = nullptr;       // [2][N] type, rank
    int* h_err = nullptr;        // pinned
    unsigned long long* trace_buf = nullptr;  // per-phase ns of k_pre (MDGB_FLAG_TRACE)
    int lb_grid = 1, lb_cap = -1, lb_ncells = -1;  // list-build launch shape for (cap, cells)
    // the other position / mirror buffer of each pair (fused NVE drift)
    double4_32a* pos_alt = nullptr;
    float4* mir_alt = nullptr;
    // coupling (host view of the per-replica settings)
    bool thermo_on = false, baro_on = false, thermo_nh = false;

    // graphs
    cudaGraphExec_t graph = nullptr;
    int graph_len = 0;
    StepParams graph_sp{};
    bool graph_valid = false;
    int64_t graph_kernels = 0;   // kernel launches one replay of the graph makes

    // stats
    mdgb_stats st{};
    std::vector<ProfEvent> prof, prof_free;

    ~mdgb_engine();
};

namespace {

int fail(mdgb_engine* e, int code, const std::string& msg) {
    if (e) e->err = msg;
    return code;
}

#define CU(call)                                                                             \
    do {                                                                                     \
        cudaError_t _e = (call);                                                             \
        if (_e != cudaSuccess)                                                               \
            return fail(e, _e == cudaErrorMemoryAllocation ? MDGB_ERR_OUT_OF_MEMORY : MDGB_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(_e));                 \
    } while (0)

template <class T>
int dalloc(mdgb_engine* e, T** p, size_t count) {
    void* q = nullptr;
    CU(cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)));
    e->allocs.push_back(q);
    *p = reinterpret_cast<T*>(q);
    return MDGB_OK;
}

void free_state(mdgb_engine* e) {
    if (e->graph) { cudaGraphExecDestroy(e->graph); e->graph = nullptr; }
    e->graph_valid = false;
    for (void* p : e->allocs) cudaFree(p);
    e->allocs.clear();
    if (e->nbr_alloc) { cudaFree(e->nbr_alloc); e->nbr_alloc = nullptr; }
    if (e->h_pin) { cudaFreeHost(e->h_pin); e->h_pin = nullptr; }
    e->has_state = false;
    e->forces_valid = false;
}

const LJ& pot_of(const mdgb_engine* e, int a, int b) {
    if (a > b) std::swap(a, b);
    return e->pot[a][b].set ? e->pot[a][b] : e->pot_default;
}

int upload_pairs(mdgb_engine* e) {
    std::vector<PairDev> tab(MAX_TYPES * MAX_TYPES);
    double fchar = 0.0;
    e->rcmax = 0.0;
    for (int a = 0; a < MAX_TYPES; ++a)
        for (int b = 0; b < MAX_TYPES; ++b) {
            const LJ& p = pot_of(e, a, b);
            PairDev q{};
            q.sigma = p.sigma; q.eps = p.eps; q.rc = p.rc; q.ucut = p.ucut;
            q.eps4 = 4.0 * p.eps;
            q.eps24 = 24.0 * p.eps;
            q.sig2f = (float)(p.sigma * p.sigma);
            q.eps4f = (float)q.eps4;
            q.eps24f = (float)q.eps24;
            q.ucutf = (float)p.ucut;
            const double rc2 = p.rc * p.rc;
            q.rc2f_lo = (float)(rc2 * (1.0 - 1e-5));
            q.rc2f_hi = (float)(rc2 * (1.0 + 1e-5));
            q.rc2_cut = sqrt_cut(p.rc);
            tab[a * MAX_TYPES + b] = q;
            if (a < e->ntypes && b < e->ntypes) {
                e->rcmax = std::max(e->rcmax, p.rc);
                fchar = std::max(fchar, std::fabs(24.0 * p.eps / p.sigma));
            }
        }
    CU(cudaMemcpyAsync((void*)e->dev.pair, tab.data(), tab.size() * sizeof(PairDev),
                       cudaMemcpyHostToDevice, e->stream));
    // fixed-point scale: a power of two putting the characteristic force near 2^31
    if (!(fchar > 0.0)) fchar = 1.0;
    const int ex = 31 - (int)std::ceil(std::log2(fchar));
    e->dev.fscale = std::ldexp(1.0f, ex);
    e->dev.fscale_log2 = ex;
    e->dev.inv_fscale = std::ldexp(1.0, -ex);
    e->dev.inv_fscale_f = std::ldexp(1.0f, -ex);
    e->skin = e->cfg.skin > 0.0 ? e->cfg.skin : 0.12 * e->rcmax;
    e->rlist = e->rcmax + e->skin;
    e->dev.rlist = e->rlist;
    e->dev.rcmax = e->rcmax;
    e->dev.skin = e->skin;
    return MDGB_OK;
}

int alloc_nbr(mdgb_engine* e, int cap) {
    // the tpa-interleaved layout (nbr_index) needs cap to be a multiple of every tpa
    cap = std::max(8, (cap + 7) & ~7);
    if (e->nbr_alloc) { cudaFree(e->nbr_alloc); e->nbr_alloc = nullptr; }
    const size_t words = (size_t)cap * (size_t)e->ntot;
    void* q = nullptr;
    CU(cudaMalloc(&q, std::max<size_t>(words, 1) * sizeof(uint32_t)));
    // a fresh list holds valid (zero) entries and zero counts until the next rebuild
    CU(cudaMemsetAsync(q, 0, std::max<size_t>(words, 1) * sizeof(uint32_t), e->stream));
    if (e->dev.nn) CU(cudaMemsetAsync(e->dev.nn, 0, (size_t)e->ntot * sizeof(int), e->stream));
    e->nbr_alloc = q;
    e->dev.nbr = reinterpret_cast<uint32_t*>(q);
    e->dev.cap = cap;
    e->cap = cap;
    e->graph_valid = false;
    return MDGB_OK;
}

void prof_begin(mdgb_engine* e, int kind, cudaEvent_t* out_b) {
    *out_b = nullptr;
    if (!(e->cfg.flags & MDGB_FLAG_PROFILE)) return;
    ProfEvent p;
    if (!e->prof_free.empty()) { p = e->prof_free.back(); e->prof_free.pop_back(); }
    else { cudaEventCreate(&p.a); cudaEventCreate(&p.b); }
    p.kind = kind;
    cudaEventRecord(p.a, e->stream);
    e->prof.push_back(p);
    *out_b = p.b;
}

void prof_end(mdgb_engine* e, cudaEvent_t b) {
    if (b) cudaEventRecord(b, e->stream);
}

void prof_collect(mdgb_engine* e) {
    for (auto& p : e->prof) {
        float ms = 0.f;
        cudaEventSynchronize(p.b);
        cudaEventElapsedTime(&ms, p.a, p.b);
        if (p.kind == 0) { e->st.force_ms += ms; e->st.force_launches++; }
        else { e->st.integrate_ms += ms; e->st.integrate_launches++; }
        e->prof_free.push_back(p);
    }
    e->prof.clear();
}

int pre_grid(const mdgb_engine* e) {
    const int maxg = std::min(4096, std::max(1, e->num_sms * e->pre_blocks_per_sm));  // bsum holds 4096
    const int want = std::max({e->ntiles, (e->ncells + 1023) / 1024, (e->nrep + TILE - 1) / TILE, 1});
    return std::min(maxg, want);
}

int launch_pre(mdgb_engine* e, const StepParams& sp) {
    cudaEvent_t pe;
    prof_begin(e, 1, &pe);
    cudaLaunchConfig_t lc{};
    lc.gridDim = dim3(pre_grid(e));
    lc.blockDim = dim3(TILE);
    lc.stream = e->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    CU(cudaLaunchKernelEx(&lc, k_pre, e->dev, sp));
    if (e->lb_cap != e->dev.cap || e->lb_ncells != e->dev.ncells) {
        e->lb_grid = list_build_grid(e->dev, e->num_sms);
        e->lb_cap = e->dev.cap;
        e->lb_ncells = e->dev.ncells;
    }
    CU(launch_list_build(e->dev, e->lb_grid, e->stream));
    prof_end(e, pe);
    e->st.kernel_launches += 2;
    return MDGB_OK;
}

// Blocks of size class c's force launch: one per tile, or (persistent) as
// many as are resident.
int force_grid(mdgb_engine* e, int c, bool kick) {
    const int ntl = e->class_ntiles[c];
    if (!(e->cfg.flags & MDGB_FLAG_PERSISTENT)) return ntl;
    const int tpa = e->class_tpa[c];
    force_fn fn = force_kernel(tpa, e->cfg.precision, e->dev.single_type != 0, kick, true, false);
    int bps = 0;
    if (!fn || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void*)fn, TILE * tpa, 0) != cudaSuccess)
        bps = 1;
    return std::min(ntl, std::max(1, bps) * e->num_sms);
}

// One force launch per non-empty size class, each with that class's threads
// per atom (the replicas of a class were listed with the same layout).
int launch_force_class(mdgb_engine* e, const StepParams& sp, bool kick, int c) {
    const bool persistent = (e->cfg.flags & MDGB_FLAG_PERSISTENT) != 0;
    const int tpa = e->class_tpa[c];
    force_fn fn = force_kernel(tpa, e->cfg.precision, e->dev.single_type != 0, kick, persistent,
                               kick && sp.fused);
    if (!fn) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "threads_per_atom must be 1, 2, 4 or 8");
    Dev d = e->dev;
    d.pos_next = e->pos_alt;
    d.mir_next = e->mir_alt;
    d.tile_list = e->dev.tile_order + e->class_tile_off[c];
    d.ntile_list = e->class_ntiles[c];
    d.list_class = c;
    const int grid = force_grid(e, c, kick);
    void* args[] = {(void*)&d, (void*)&sp};
    CU(cudaLaunchKernel((const void*)fn, dim3(grid), dim3(TILE * tpa), args, 0, e->stream));
    e->st.kernel_launches++;
    return MDGB_OK;
}

int launch_force(mdgb_engine* e, const StepParams& sp_in, bool kick) {
    cudaEvent_t pe;
    prof_begin(e, 0, &pe);
    if (e->cfg.flags & MDGB_FLAG_PERSISTENT)
        CU(cudaMemsetAsync(e->dev.queue, 0, mdgb_engine::NCLASS * sizeof(unsigned int), e->stream));
    const StepParams& sp = sp_in;
    band_fn bk = band_kernel(e->cfg.precision);
    if (bk) CU(cudaMemsetAsync(e->dev.band_count, 0, sizeof(int), e->stream));
    for (int c = 0; c < mdgb_engine::NCLASS; ++c) {
        if (!e->class_ntiles[c]) continue;
        int rc = launch_force_class(e, sp, kick, c);
        if (rc) return rc;
    }
    if (bk) {
        // the atoms the force launches left: same buffers as they used
        Dev d = e->dev;
        d.pos_next = e->pos_alt;
        d.mir_next = e->mir_alt;
        int kk = kick ? 1 : 0;
        void* args[] = {(void*)&d, (void*)&sp, (void*)&kk};
        CU(cudaLaunchKernel((const void*)bk, dim3(4 * e->num_sms), dim3(128), args, 0, e->stream));
        e->st.kernel_launches++;
    }
    prof_end(e, pe);
    if (kick && sp.fused) {   // the next positions/mirrors are in the other buffers now
        std::swap(e->dev.pos, e->pos_alt);
        std::swap(e->dev.mir, e->mir_alt);
    }
    return MDGB_OK;
}

// Write the per-replica threads per atom (the list layout) of every size class.
int apply_class_tpa(mdgb_engine* e) {
    CU(cudaMemcpyAsync(e->rep_host.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    for (int r = 0; r < e->nrep; ++r) e->rep_host[r].tpa = e->class_tpa[e->class_of[r]];
    CU(cudaMemcpyAsync(e->dev.rep, e->rep_host.data(), e->nrep * sizeof(RepDev), cudaMemcpyHostToDevice, e->stream));
    e->graph_valid = false;
    return MDGB_OK;
}

StepParams make_sp(const mdgb_engine* e, double dt, bool drift) {
    StepParams sp{};
    sp.dt = dt;
    for (int t = 0; t < MAX_TYPES; ++t)
        sp.kick_c[t] = t < (int)e->mass.size() ? dt / (2.0 * e->mass[t]) : 0.0;  // integrator.rs:29-30
    sp.coupled = (e->thermo_on || e->baro_on) ? 1 : 0;
    sp.thermo_nh = e->thermo_nh ? 1 : 0;
    sp.fixed_interval = e->cfg.rebuild_every;
    sp.force_rebuild = 0;
    sp.do_drift = drift ? 1 : 0;
    return sp;
}

int read_err(mdgb_engine* e, int* flags) {
    CU(cudaMemcpyAsync(e->h_err, e->dev.err, 2 * sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    *flags = e->h_err[0];
    return MDGB_OK;
}

int clear_err(mdgb_engine* e) {
    CU(cudaMemsetAsync(e->dev.err, 0, 2 * sizeof(int), e->stream));
    CU(cudaMemsetAsync(e->dev.bar, 0, 4 * sizeof(unsigned int), e->stream));
    return MDGB_OK;
}

int snapshot(mdgb_engine* e, bool restore) {
    const size_t N = e->ntot;
    auto cp = [&](void* dst, const void* src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, e->stream);
    };
    Dev& d = e->dev;
    if (!restore) {
        CU(cp(e->snap_pos, d.pos, N * sizeof(double4_32a)));
        CU(cp(e->snap_d, d.vel, 3 * N * sizeof(double)));
        CU(cp(e->snap_d + 3 * N, d.frc, 3 * N * sizeof(double)));
        CU(cp(e->snap_d + 6 * N, d.epot, N * sizeof(double)));
        CU(cp(e->snap_d + 7 * N, d.evir, N * sizeof(double)));
        CU(cp(e->snap_i, d.orig, N * sizeof(int)));
        CU(cp(e->snap_i + N, d.rank, N * sizeof(int)));
        CU(cp(e->snap_i + 2 * N, d.cell, N * sizeof(int)));
        CU(cp(e->snap_i + 3 * N, d.slot_of_rank, N * sizeof(int)));
        CU(cp(e->snap_mir0, d.mir0, N * sizeof(float4)));
        CU(cp(e->snap_rep, d.rep, e->nrep * sizeof(RepDev)));
    } else {
        CU(cp(d.pos, e->snap_pos, N * sizeof(double4_32a)));
        CU(cp(d.vel, e->snap_d, 3 * N * sizeof(double)));
        CU(cp(d.frc, e->snap_d + 3 * N, 3 * N * sizeof(double)));
        CU(cp(d.epot, e->snap_d + 6 * N, N * sizeof(double)));
        CU(cp(d.evir, e->snap_d + 7 * N, N * sizeof(double)));
        CU(cp(d.orig, e->snap_i, N * sizeof(int)));
        CU(cp(d.rank, e->snap_i + N, N * sizeof(int)));
        CU(cp(d.cell, e->snap_i + 2 * N, N * sizeof(int)));
        CU(cp(d.slot_of_rank, e->snap_i + 3 * N, N * sizeof(int)));
        CU(cp(d.mir0, e->snap_mir0, N * sizeof(float4)));
        CU(cp(d.rep, e->snap_rep, e->nrep * sizeof(RepDev)));
    }
    return MDGB_OK;
}

int grow_list(mdgb_engine* e) {
    int needed = 0;
    CU(cudaMemcpyAsync(&needed, e->dev.max_needed, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    int cap = std::max(e->cap + 8, (int)std::ceil(needed * 1.25));
    cap = (cap + 7) & ~7;
    CU(cudaMemsetAsync(e->dev.max_needed, 0, sizeof(int), e->stream));
    int rc = alloc_nbr(e, cap);
    if (rc) return rc;
    e->st.neighbor_capacity = cap;
    return MDGB_OK;
}

// Forced rebuild + mirror refresh without integration.
int refresh(mdgb_engine* e, bool force_rebuild) {
    StepParams sp = make_sp(e, 0.0, false);
    sp.force_rebuild = force_rebuild ? 1 : 0;
    return launch_pre(e, sp);
}

int check_flags(mdgb_engine* e, int flags) {
    if (flags & E_TIMEOUT) return fail(e, MDGB_ERR_DEVICE_TIMEOUT, "a device-side grid barrier timed out");
    if (flags & E_FIXED)
        return fail(e, MDGB_ERR_FIXED_POINT_OVERFLOW,
                    "a pair force left the 64-bit fixed-point range (atoms overlapping?)");
    if (flags & (E_BOUNDS | E_CELLS)) return fail(e, MDGB_ERR_CUDA, "internal index check failed");
    return MDGB_OK;
}

int compute_forces_impl(mdgb_engine* e) {
    for (int attempt = 0; attempt < 8; ++attempt) {
        int rc = clear_err(e);
        if (rc) return rc;
        rc = refresh(e, true);
        if (rc) return rc;
        StepParams sp = make_sp(e, 0.0, false);
        rc = launch_force(e, sp, false);
        if (rc) return rc;
        int flags = 0;
        rc = read_err(e, &flags);
        if (rc) return rc;
        if (flags & E_NLIST) {
            rc = grow_list(e);
            if (rc) return rc;
            e->st.retries++;
            continue;
        }
        return check_flags(e, flags);
    }
    return fail(e, MDGB_ERR_NEIGHBOR_OVERFLOW, "neighbour list kept overflowing");
}

// n steps.  NVE chunks fuse each step's first kick and drift into the force
// pass of the step before (steps 2..nf+1); nf is even, so the position/mirror
// buffer pair ends the chunk the way round it started (a captured graph stays
// valid), and the chunk's last step is unfused, leaving the state at a whole
// step.
int run_chunk_kernels(mdgb_engine* e, const StepParams& sp, int n) {
    const bool fusable = sp.do_drift && !sp.coupled && !sp.thermo_nh;
    const int nf = fusable ? ((n - 1) & ~1) : 0;
    for (int i = 0; i < n; ++i) {
        StepParams pre = sp;
        pre.predrifted = (i >= 1 && i <= nf) ? 1 : 0;
        int rc = launch_pre(e, pre);
        if (rc) return rc;
        StepParams frc = sp;
        frc.fused = i < nf ? 1 : 0;
        rc = launch_force(e, frc, true);
        if (rc) return rc;
    }
    return MDGB_OK;
}

bool same_sp(const StepParams& a, const StepParams& b) { return std::memcmp(&a, &b, sizeof(a)) == 0; }

int run_chunk(mdgb_engine* e, const StepParams& sp, int n) {
    const bool use_graph = e->cfg.graph_steps > 1 && !(e->cfg.flags & MDGB_FLAG_PROFILE) &&
                           n == e->cfg.graph_steps;
    if (!use_graph) return run_chunk_kernels(e, sp, n);
    if (!e->graph_valid || e->graph_len != n || !same_sp(e->graph_sp, sp)) {
        if (e->graph) { cudaGraphExecDestroy(e->graph); e->graph = nullptr; }
        cudaGraph_t g = nullptr;
        CU(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        const int64_t launches0 = e->st.kernel_launches;
        // capture runs nothing: the buffer pair must read as before afterwards
        double4_32a* const pos0 = e->dev.pos; double4_32a* const pos1 = e->pos_alt;
        float4* const mir0 = e->dev.mir; float4* const mir1 = e->mir_alt;
        int rc = run_chunk_kernels(e, sp, n);
        cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
        e->dev.pos = pos0; e->pos_alt = pos1; e->dev.mir = mir0; e->mir_alt = mir1;
        e->graph_kernels = e->st.kernel_launches - launches0;
        e->st.kernel_launches = launches0;
        if (rc || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            e->cfg.graph_steps = 0;  // capture unsupported here: stay eager
            return run_chunk_kernels(e, sp, n);
        }
        ce = cudaGraphInstantiate(&e->graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            cudaGetLastError();
            e->cfg.graph_steps = 0;
            return run_chunk_kernels(e, sp, n);
        }
        e->graph_valid = true;
        e->graph_len = n;
        e->graph_sp = sp;
    }
    CU(cudaGraphLaunch(e->graph, e->stream));
    e->st.graph_launches++;
    e->st.kernel_launches += e->graph_kernels;
    return MDGB_OK;
}

int autotune_tpa(mdgb_engine* e);

int step_impl(mdgb_engine* e, int64_t nsteps, double dt) {
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    if (nsteps < 0 || !(dt == dt)) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "bad nsteps or dt");
    if (!e->tuned) {
        int rc = autotune_tpa(e);
        if (rc) return rc;
    }
    const StepParams sp = make_sp(e, dt, true);
    const int chunk = e->cfg.graph_steps > 1 ? e->cfg.graph_steps : 64;
    int64_t done = 0;
    int retries = 0;
    while (done < nsteps) {
        const int n = (int)std::min<int64_t>(chunk, nsteps - done);
        int rc = clear_err(e);
        if (rc) return rc;
        rc = snapshot(e, false);
        if (rc) return rc;
        rc = run_chunk(e, sp, n);
        if (rc) return rc;
        int flags = 0;
        rc = read_err(e, &flags);
        if (rc) return rc;
        if (flags & E_NLIST) {
            if (++retries > 8) return fail(e, MDGB_ERR_NEIGHBOR_OVERFLOW, "neighbour list kept overflowing");
            rc = grow_list(e);
            if (rc) return rc;
            rc = snapshot(e, true);
            if (rc) return rc;
            // the restored state keeps its cells; rebuild lists at the new capacity
            rc = clear_err(e);
            if (rc) return rc;
            rc = refresh(e, true);
            if (rc) return rc;
            e->st.retries++;
            continue;
        }
        rc = check_flags(e, flags);
        if (rc) return rc;
        done += n;
        e->st.steps += n;
    }
    // finish the last step's barostat update (barostat.rs:45-48)
    if (e->baro_on) {
        void* args[] = {(void*)&e->dev};
        CU(cudaLaunchKernel((const void*)k_apply_pending, dim3(e->ntiles), dim3(TILE), args, 0, e->stream));
        CU(cudaLaunchKernel((const void*)k_apply_pending_box, dim3((e->nrep + 127) / 128), dim3(128), args, 0,
                            e->stream));
        e->st.kernel_launches += 2;
    }
    e->forces_valid = true;
    return MDGB_OK;
}

// Threads per atom for each size class: every candidate is timed on every
// class at once (each class's launch bracketed by its own events), and each
// class keeps its fastest.
int autotune_tpa(mdgb_engine* e) {
    e->tuned = true;
    const int NC = mdgb_engine::NCLASS;
    if (e->dev.refmode || e->cfg.threads_per_atom > 0) {
        const int t = e->dev.refmode ? 1 : e->cfg.threads_per_atom;
        for (int c = 0; c < NC; ++c) e->class_tpa[c] = t;
        e->tpa = t;
        int rc = apply_class_tpa(e);
        if (rc) return rc;
        return refresh(e, true);
    }
    // Keep the caller's forces: tuning evaluates forces into scratch.
    const size_t N = e->ntot;
    CU(cudaMemcpyAsync(e->snap_d, e->dev.frc, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
    CU(cudaMemcpyAsync(e->snap_d + 3 * N, e->dev.epot, N * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
    CU(cudaMemcpyAsync(e->snap_d + 4 * N, e->dev.evir, N * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
    const int cands[4] = {1, 2, 4, 8};
    float best[NC];
    int best_tpa[NC];
    for (int c = 0; c < NC; ++c) { best[c] = 1e30f; best_tpa[c] = 1; }
    cudaEvent_t ev[NC][2];
    for (int c = 0; c < NC; ++c) { CU(cudaEventCreate(&ev[c][0])); CU(cudaEventCreate(&ev[c][1])); }
    const unsigned saved_flags = e->cfg.flags;
    e->cfg.flags &= ~(MDGB_FLAG_PROFILE | MDGB_FLAG_PERSISTENT);
    StepParams sp = make_sp(e, 0.0, false);
    int rc = MDGB_OK;
    for (int ci = 0; ci < 4 && !rc; ++ci) {
        const int cand = cands[ci];
        if (e->ntot < 4096 && cand > 1) break;  // tiny systems: not worth measuring
        for (int c = 0; c < NC; ++c) e->class_tpa[c] = cand;
        rc = apply_class_tpa(e);
        if (!rc) rc = clear_err(e);
        if (!rc) rc = refresh(e, true);
        if (!rc) rc = launch_force(e, sp, false);  // warm-up
        if (rc) break;
        for (int c = 0; c < NC && !rc; ++c) {
            if (!e->class_ntiles[c]) continue;
            CU(cudaEventRecord(ev[c][0], e->stream));
            for (int i = 0; i < 3 && !rc; ++i) rc = launch_force_class(e, sp, false, c);
            CU(cudaEventRecord(ev[c][1], e->stream));
        }
        if (rc) break;
        int flags = 0;
        rc = read_err(e, &flags);
        if (rc) break;
        if (flags & E_NLIST) {
            rc = grow_list(e);
            if (!rc) rc = clear_err(e);
            --ci;  // same candidate again with the larger list
            continue;
        }
        for (int c = 0; c < NC; ++c) {
            if (!e->class_ntiles[c]) continue;
            float ms = 0.f;
            CU(cudaEventElapsedTime(&ms, ev[c][0], ev[c][1]));
            if (ms < best[c]) { best[c] = ms; best_tpa[c] = cand; }
        }
    }
    e->cfg.flags = saved_flags;
    for (int c = 0; c < NC; ++c) { cudaEventDestroy(ev[c][0]); cudaEventDestroy(ev[c][1]); }
    if (rc) return rc;
    for (int c = 0; c < NC; ++c) e->class_tpa[c] = best_tpa[c];
    e->tpa = best_tpa[0];
    for (int c = NC - 1; c >= 0; --c)
        if (e->class_ntiles[c]) { e->tpa = best_tpa[c]; break; }
    e->st.threads_per_atom = e->tpa;
    CU(cudaMemcpyAsync(e->dev.frc, e->snap_d, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
    CU(cudaMemcpyAsync(e->dev.epot, e->snap_d + 3 * N, N * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
    CU(cudaMemcpyAsync(e->dev.evir, e->snap_d + 4 * N, N * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
    rc = apply_class_tpa(e);
    if (!rc) rc = clear_err(e);
    if (rc) return rc;
    return refresh(e, true);  // lists in the chosen layouts
}

int upload_impl(mdgb_engine* e, int nrep, const int64_t* offsets, const uint16_t* type, const double* pos,
                const double* vel, const double* mass_per_type, int ntypes, const double* boxes) {
    if (nrep < 1 || !offsets || !type || !pos || !mass_per_type || !boxes)
        return fail(e, MDGB_ERR_INVALID_ARGUMENT, "null argument");
    if (ntypes < 1 || ntypes > MAX_TYPES)
        return fail(e, MDGB_ERR_INVALID_ARGUMENT, "ntypes must be in 1..16");
    const int64_t n = offsets[nrep];
    if (offsets[0] != 0 || n < 1 || n >= (int64_t)IDX_MASK)
        return fail(e, MDGB_ERR_INVALID_ARGUMENT, "bad offsets / atom count");
    for (int r = 0; r < nrep; ++r) {
        if (offsets[r + 1] <= offsets[r]) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "empty replica");
        for (int a = 0; a < 3; ++a)
            if (!(boxes[3 * r + a] > 0.0)) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "box must be positive");
    }
    for (int t = 0; t < ntypes; ++t)
        if (!(mass_per_type[t] > 0.0)) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "mass must be positive");
    free_state(e);
    e->ntot = (int)n;
    e->nrep = nrep;
    e->ntypes = ntypes;
    e->offsets.assign(offsets, offsets + nrep + 1);
    e->mass.assign(mass_per_type, mass_per_type + ntypes);
    const int N = e->ntot;

    // reference ranks (type-major within each replica) and per-replica type offsets
    std::vector<int> rank(N), itype(N);
    e->rep_host.assign(nrep, RepDev{});
    for (int r = 0; r < nrep; ++r) {
        std::vector<int64_t> cnt(ntypes + 1, 0);
        for (int64_t i = offsets[r]; i < offsets[r + 1]; ++i) {
            if (type[i] >= ntypes) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "type id >= ntypes");
            cnt[type[i] + 1]++;
        }
        for (int t = 0; t < ntypes; ++t)
            if (cnt[t + 1] == 0)
                return fail(e, MDGB_ERR_INVALID_ARGUMENT,
                            "every type 0..ntypes-1 needs at least one atom in every replica "
                            "(the reference indexes particles[type][0])");
        for (int t = 0; t < ntypes; ++t) cnt[t + 1] += cnt[t];
        RepDev& R = e->rep_host[r];
        for (int t = 0; t <= ntypes; ++t) R.type_off[t] = (int)cnt[t];
        for (int t = ntypes + 1; t <= MAX_TYPES; ++t) R.type_off[t] = (int)cnt[ntypes];
        std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
        for (int64_t i = offsets[r]; i < offsets[r + 1]; ++i) {
            rank[i] = (int)(offsets[r] + fill[type[i]]++);
            itype[i] = type[i];
        }
        R.last_type_count = (int)(cnt[ntypes] - cnt[ntypes - 1]);
    }

    // potentials, list radius
    int rc = dalloc(e, (PairDev**)&e->dev.pair, MAX_TYPES * MAX_TYPES);
    if (rc) return rc;
    e->dev.ntypes = ntypes;
    rc = upload_pairs(e);
    if (rc) return rc;

    // tiles and cells
    std::vector<int4> tiles;
    std::vector<int> cell_rep;
    int max_rep_n = 0;
    double max_density = 0.0;
    for (int r = 0; r < nrep; ++r) {
        RepDev& R = e->rep_host[r];
        const int nr = (int)(offsets[r + 1] - offsets[r]);
        max_rep_n = std::max(max_rep_n, nr);
        R.begin = offsets[r];
        R.n = nr;
        R.tile_begin = (int)tiles.size();
        for (int b = 0; b < nr; b += TILE) tiles.push_back(make_int4(r, (int)(offsets[r] + b), std::min(TILE, nr - b), 0));
        R.ntiles = (int)tiles.size() - R.tile_begin;
        double prod = 1.0;
        for (int a = 0; a < 3; ++a) {
            const double L = boxes[3 * r + a];
            R.box[a] = L; R.box_build[a] = L; R.cs[a] = L; R.inv_cs[a] = 1.0 / L; R.nc[a] = 1;
            prod *= std::max(1.0, std::floor(L / (e->rlist * (1.0 + 1e-6))));
        }
        const double vol = boxes[3 * r] * boxes[3 * r + 1] * boxes[3 * r + 2];
        max_density = std::max(max_density, nr / vol);
        const double capd = std::min(std::ceil(prod * 1.3) + 27.0, 2.0 * nr + 27.0);
        R.cell_cap = (int)std::max(27.0, capd);
        R.cell_base = (int)cell_rep.size();
        cell_rep.insert(cell_rep.end(), R.cell_cap, r);
        R.mode = MODE_BRUTE;
        R.pending = 1.0;
        R.lambda = 0.0;
        R.myu = 0.0;
        R.rebuild = 1;
    }
    e->ntiles = (int)tiles.size();
    e->ncells = (int)cell_rep.size();
    // reduction chunks: runs of <= CHUNK_TILES tiles inside one replica
    std::vector<int4> chunks;
    for (int r = 0; r < nrep; ++r) {
        RepDev& R = e->rep_host[r];
        R.chunk_begin = (int)chunks.size();
        for (int t = 0; t < R.ntiles; t += CHUNK_TILES)
            chunks.push_back(make_int4(r, R.tile_begin + t, std::min(CHUNK_TILES, R.ntiles - t), 0));
        R.nchunks = (int)chunks.size() - R.chunk_begin;
    }

    Dev& d = e->dev;
    d.ntot = N; d.ntiles = e->ntiles; d.nrep = nrep; d.ncells = e->ncells;
    d.refmode = (e->cfg.flags & MDGB_FLAG_REFERENCE_ORDER) && e->cfg.precision == MDGB_PRECISION_FP64 ? 1 : 0;
    d.mixed = e->cfg.precision != MDGB_PRECISION_FP64 ? 1 : 0;
    d.single_type = ntypes == 1 ? 1 : 0;
    d.last_type = ntypes - 1;
    for (int t = 0; t < MAX_TYPES; ++t) d.mass[t] = t < ntypes ? mass_per_type[t] : 1.0;

    if ((rc = dalloc(e, &d.pos, N)) || (rc = dalloc(e, &d.vel, 3 * (size_t)N)) ||
        (rc = dalloc(e, &d.frc, 3 * (size_t)N)) || (rc = dalloc(e, &d.epot, N)) ||
        (rc = dalloc(e, &d.evir, N)) || (rc = dalloc(e, &d.mir, N)) || (rc = dalloc(e, &d.mir0, N)) ||
        (rc = dalloc(e, &e->pos_alt, N)) || (rc = dalloc(e, &e->mir_alt, N)) ||
        (rc = dalloc(e, &d.band_list, N)) || (rc = dalloc(e, &d.band_count, 1)) ||
        (rc = dalloc(e, &d.cell, N)) || (rc = dalloc(e, &d.orig, N)) || (rc = dalloc(e, &d.rank, N)) ||
        (rc = dalloc(e, &d.nn, N)) || (rc = dalloc(e, &d.tiles, e->ntiles)) ||
        (rc = dalloc(e, &d.rep, nrep)) || (rc = dalloc(e, &d.part, 8 * (size_t)e->ntiles)) ||
        (rc = dalloc(e, &d.cpart, 8 * chunks.size())) || (rc = dalloc(e, &d.chunks, chunks.size())) ||
        (rc = dalloc(e, &d.err, 2)) || (rc = dalloc(e, &d.max_needed, 1)) ||
        (rc = dalloc(e, &d.cell_count, e->ncells)) ||
        (rc = dalloc(e, &d.cell_start, e->ncells + 1)) || (rc = dalloc(e, &d.cell_rep, e->ncells)) ||
        (rc = dalloc(e, &d.perm, N)) || (rc = dalloc(e, &d.tmp_pos, N)) ||
        (rc = dalloc(e, &d.tmp_d, 8 * (size_t)N)) || (rc = dalloc(e, &d.tmp_i, 4 * (size_t)N)) ||
        (rc = dalloc(e, &d.slot_of_rank, N)) || (rc = dalloc(e, &d.bsum, 4096)) ||
        (rc = dalloc(e, &d.bar, 4)) || (rc = dalloc(e, &d.queue, mdgb_engine::NCLASS)) ||
        (rc = dalloc(e, &e->trace_buf, TR_SLOTS)) ||
        (rc = dalloc(e, &d.tile_order, e->ntiles)) ||
        (rc = dalloc(e, &e->snap_pos, N)) || (rc = dalloc(e, &e->snap_d, 8 * (size_t)N)) ||
        (rc = dalloc(e, &e->snap_i, 4 * (size_t)N)) || (rc = dalloc(e, &e->snap_mir0, N)) ||
        (rc = dalloc(e, &e->snap_rep, nrep)) || (rc = dalloc(e, &e->d_out, 11 * (size_t)N)) ||
        (rc = dalloc(e, &e->d_in_i, 2 * (size_t)N)))
        return rc;
    CU(cudaMallocHost((void**)&e->h_pin, 11 * (size_t)N * sizeof(double)));
    if (!e->h_err) CU(cudaMallocHost((void**)&e->h_err, 4 * sizeof(int)));

    // neighbour capacity from the densest replica (grows on overflow)
    int cap = e->cfg.neighbor_capacity;
    if (cap <= 0) {
        const double expect = 4.0 / 3.0 * M_PI * std::pow(e->rlist * (1.0 + 1e-5), 3) * max_density;
        cap = (int)std::ceil(expect * 1.35 + 16.0);
        cap = std::min(cap, std::max(max_rep_n - 1, 8));
    }
    cap = std::max(8, (cap + 7) & ~7);
    rc = alloc_nbr(e, cap);
    if (rc) return rc;
    e->st = mdgb_stats{};
    e->st.neighbor_capacity = cap;

    // tile order for the persistent kernel: costliest (densest replica) first
    std::vector<int> order(e->ntiles);
    for (int i = 0; i < e->ntiles; ++i) order[i] = i;
    std::vector<double> cost(e->ntiles);
    for (int i = 0; i < e->ntiles; ++i) {
        const RepDev& R = e->rep_host[tiles[i].x];
        const double vol = R.box[0] * R.box[1] * R.box[2];
        const double dens = R.n / vol;
        cost[i] = tiles[i].z * std::min((double)R.n, 1.0 + dens * 4.0 / 3.0 * M_PI * std::pow(e->rlist, 3));
    }
    // size classes by replica atom count; tile_order = class 0 tiles, class 1, class 2
    e->class_of.assign(nrep, 0);
    for (int c = 0; c < mdgb_engine::NCLASS; ++c) { e->class_ntiles[c] = 0; e->class_nrep[c] = 0; }
    for (int r = 0; r < nrep; ++r) {
        const int nr = e->rep_host[r].n;
        const int c = nr < 2048 ? 0 : (nr < 32768 ? 1 : 2);
        e->class_of[r] = c;
        e->rep_host[r].size_class = c;
        e->class_nrep[c]++;
        e->class_ntiles[c] += e->rep_host[r].ntiles;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const int ca = e->class_of[tiles[a].x], cb = e->class_of[tiles[b].x];
        if (ca != cb) return ca < cb;
        return cost[a] > cost[b];
    });
    e->class_tile_off[0] = 0;
    for (int c = 1; c < mdgb_engine::NCLASS; ++c) e->class_tile_off[c] = e->class_tile_off[c - 1] + e->class_ntiles[c - 1];

    CU(cudaMemcpyAsync(d.tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, e->stream));
    d.nchunks = (int)chunks.size();
    CU(cudaMemcpyAsync(d.chunks, chunks.data(), chunks.size() * sizeof(int4), cudaMemcpyHostToDevice, e->stream));
    CU(cudaMemcpyAsync(d.tile_order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    CU(cudaMemcpyAsync(d.cell_rep, cell_rep.data(), cell_rep.size() * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    CU(cudaMemsetAsync(d.cell_count, 0, e->ncells * sizeof(int), e->stream));
    CU(cudaMemsetAsync(d.max_needed, 0, sizeof(int), e->stream));
    CU(cudaMemsetAsync(e->trace_buf, 0, TR_SLOTS * sizeof(unsigned long long), e->stream));
    d.trace = (e->cfg.flags & MDGB_FLAG_TRACE) ? e->trace_buf : nullptr;
    CU(cudaMemsetAsync(d.err, 0, 2 * sizeof(int), e->stream));
    CU(cudaMemsetAsync(d.bar, 0, 4 * sizeof(unsigned int), e->stream));
    {
        const int t0 = (e->cfg.flags & MDGB_FLAG_REFERENCE_ORDER) && e->cfg.precision == MDGB_PRECISION_FP64
                           ? 1 : (e->cfg.threads_per_atom > 0 ? e->cfg.threads_per_atom : 1);
        for (int c = 0; c < mdgb_engine::NCLASS; ++c) e->class_tpa[c] = t0;
        for (int r = 0; r < nrep; ++r) e->rep_host[r].tpa = t0;
    }
    CU(cudaMemcpyAsync(d.rep, e->rep_host.data(), nrep * sizeof(RepDev), cudaMemcpyHostToDevice, e->stream));
    // staging copies of the caller's arrays
    double* dpos = e->d_out;
    double* dvel = e->d_out + 3 * (size_t)N;
    std::memcpy(e->h_pin, pos, 3 * (size_t)N * sizeof(double));
    if (vel) std::memcpy(e->h_pin + 3 * (size_t)N, vel, 3 * (size_t)N * sizeof(double));
    CU(cudaMemcpyAsync(dpos, e->h_pin, (vel ? 6 : 3) * (size_t)N * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    int* hi = reinterpret_cast<int*>(e->h_pin + 6 * (size_t)N);
    CU(cudaStreamSynchronize(e->stream));
    std::memcpy(hi, itype.data(), N * sizeof(int));
    std::memcpy(hi + N, rank.data(), N * sizeof(int));
    CU(cudaMemcpyAsync(e->d_in_i, hi, 2 * (size_t)N * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    const double* vptr = vel ? dvel : nullptr;
    const int* tptr = e->d_in_i;
    const int* rptr = e->d_in_i + N;
    void* args[] = {(void*)&e->dev, (void*)&dpos, (void*)&vptr, (void*)&tptr, (void*)&rptr};
    CU(cudaLaunchKernel((const void*)k_scatter_in, dim3((N + 255) / 256), dim3(256), args, 0, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    e->has_state = true;
    e->forces_valid = false;
    e->thermo_on = e->baro_on = e->thermo_nh = false;
    e->tuned = false;
    e->tpa = e->class_tpa[0];
    d.tpa = e->tpa;
    // bin and build lists now, so a bare mdgb_step starts from a valid list
    rc = clear_err(e);
    if (rc) return rc;
    rc = refresh(e, true);
    if (rc) return rc;
    int flags = 0;
    rc = read_err(e, &flags);
    if (rc) return rc;
    if (flags & E_NLIST) {
        rc = grow_list(e);
        if (rc) return rc;
        rc = clear_err(e);
        if (!rc) rc = refresh(e, true);
        if (rc) return rc;
        rc = read_err(e, &flags);
        if (rc) return rc;
    }
    return check_flags(e, flags & ~E_NLIST);
}

int set_coupling_impl(mdgb_engine* e, const mdgb_thermostat* th, const mdgb_barostat* ba) {
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    CU(cudaMemcpyAsync(e->rep_host.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    bool any_nh = false;
    for (int r = 0; r < e->nrep; ++r) {
        RepDev& R = e->rep_host[r];
        R.thermo_on = th ? 1 : 0;
        if (th) {
            if (th[r].kind != MDGB_THERMOSTAT_BERENDSEN && th[r].kind != MDGB_THERMOSTAT_NOSE_HOOVER)
                return fail(e, MDGB_ERR_INVALID_ARGUMENT, "unknown thermostat kind");
            if (th[r].kind == MDGB_THERMOSTAT_NOSE_HOOVER) any_nh = true;
            R.thermo_kind = th[r].kind;
            R.th_tau = th[r].tau; R.th_T0 = th[r].target_temperature;
            R.lambda = th[r].lambda; R.psi = th[r].psi;
        }
        R.baro_on = ba ? 1 : 0;
        if (ba) {
            R.ba_beta = ba[r].beta; R.ba_tau = ba[r].tau; R.ba_P0 = ba[r].target_pressure;
            R.myu = ba[r].myu;
        }
    }
    if (any_nh && e->ntypes > 1)
        return fail(e, MDGB_ERR_UNSUPPORTED,
                    "Nose-Hoover coupling is implemented for single-type systems (the reference's per-type "
                    "psi accumulation across several types is not)");
    e->thermo_nh = any_nh;
    e->thermo_on = th != nullptr;
    e->baro_on = ba != nullptr;
    CU(cudaMemcpyAsync(e->dev.rep, e->rep_host.data(), e->nrep * sizeof(RepDev), cudaMemcpyHostToDevice, e->stream));
    return MDGB_OK;
}

int get_coupling_impl(mdgb_engine* e, mdgb_thermostat* th, mdgb_barostat* ba) {
    CU(cudaMemcpyAsync(e->rep_host.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    for (int r = 0; r < e->nrep; ++r) {
        const RepDev& R = e->rep_host[r];
        if (th) { th[r].lambda = R.lambda; th[r].psi = R.psi; }
        if (ba) ba[r].myu = R.myu;
    }
    return MDGB_OK;
}

int download_impl(mdgb_engine* e, double* pos, double* vel, double* force, double* pot, double* temp,
                  double* boxes) {
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    const size_t N = e->ntot;
    double* o = e->d_out;
    double *op = o, *ov = o + 3 * N, *of = o + 6 * N, *oe = o + 9 * N, *ot = o + 10 * N;
    void* args[] = {(void*)&e->dev, (void*)&op, (void*)&ov, (void*)&of, (void*)&oe, (void*)&ot};
    CU(cudaLaunchKernel((const void*)k_gather_out, dim3((unsigned)((N + 255) / 256)), dim3(256), args, 0, e->stream));
    CU(cudaMemcpyAsync(e->h_pin, e->d_out, 11 * N * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaMemcpyAsync(e->rep_host.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    if (pos) std::memcpy(pos, e->h_pin, 3 * N * sizeof(double));
    if (vel) std::memcpy(vel, e->h_pin + 3 * N, 3 * N * sizeof(double));
    if (force) std::memcpy(force, e->h_pin + 6 * N, 3 * N * sizeof(double));
    if (pot) std::memcpy(pot, e->h_pin + 9 * N, N * sizeof(double));
    if (temp) std::memcpy(temp, e->h_pin + 10 * N, N * sizeof(double));
    if (boxes)
        for (int r = 0; r < e->nrep; ++r)
            for (int a = 0; a < 3; ++a) boxes[3 * r + a] = e->rep_host[r].box[a];
    return MDGB_OK;
}

int macro_impl(mdgb_engine* e, int type, mdgb_macro* out) {
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    if (type < 0 || type >= e->ntypes) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "type out of range");
    if (!out) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "null output");
    int rc = clear_err(e);
    if (rc) return rc;
    StepParams sp = make_sp(e, 0.0, false);
    cudaLaunchConfig_t lc{};
    lc.gridDim = dim3(pre_grid(e));
    lc.blockDim = dim3(TILE);
    lc.stream = e->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    CU(cudaLaunchKernelEx(&lc, k_macro, e->dev, sp, type));
    e->st.kernel_launches++;
    int flags = 0;
    rc = read_err(e, &flags);
    if (rc) return rc;
    rc = check_flags(e, flags);
    if (rc) return rc;
    CU(cudaMemcpyAsync(e->rep_host.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    for (int r = 0; r < e->nrep; ++r) {
        const RepDev& R = e->rep_host[r];
        mdgb_macro& m = out[r];
        m.kinetic_energy = R.ke;
        m.potential_energy = R.pe;
        m.thermal_energy = R.thermal;
        m.temperature = R.T;
        m.pressure = R.P;
        for (int a = 0; a < 3; ++a) { m.com_velocity[a] = R.vcm[a]; m.momentum[a] = R.mom[a]; }
        m.count = R.count;
    }
    return MDGB_OK;
}

}  // namespace

mdgb_engine::~mdgb_engine() {
    free_state(this);
    for (auto& p : prof) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto& p : prof_free) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    if (h_err) cudaFreeHost(h_err);
    if (stream) cudaStreamDestroy(stream);
}

// ===========================================================================
extern "C" {

MDGB_API int mdgb_abi_version(void) { return MDGB_ABI_VERSION; }

MDGB_API int mdgb_config_default(mdgb_config* cfg) {
    if (!cfg) return MDGB_ERR_INVALID_ARGUMENT;
    *cfg = mdgb_config{};
    cfg->precision = MDGB_PRECISION_MIXED;
    cfg->skin = 0.0;
    cfg->rebuild_every = 0;
    cfg->threads_per_atom = 0;
    cfg->graph_steps = 0;
    cfg->neighbor_capacity = 0;
    cfg->device = 0;
    cfg->flags = 0;
    return MDGB_OK;
}

MDGB_API int mdgb_create(const mdgb_config* cfg, mdgb_engine** out) {
    if (!out) return MDGB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    mdgb_config c;
    if (cfg) c = *cfg; else mdgb_config_default(&c);
    if (c.precision != MDGB_PRECISION_FP64 && c.precision != MDGB_PRECISION_MIXED &&
        c.precision != MDGB_PRECISION_FP32_NAIVE)
        return MDGB_ERR_INVALID_ARGUMENT;
    if (c.threads_per_atom != 0 && c.threads_per_atom != 1 && c.threads_per_atom != 2 &&
        c.threads_per_atom != 4 && c.threads_per_atom != 8)
        return MDGB_ERR_INVALID_ARGUMENT;
    if ((c.flags & MDGB_FLAG_REFERENCE_ORDER) && c.precision == MDGB_PRECISION_FP64) c.threads_per_atom = 1;
    mdgb_engine* e = new mdgb_engine();
    e->cfg = c;
    e->device = c.device;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        delete e;
        return MDGB_ERR_CUDA;
    }
    if (cudaSetDevice(c.device) != cudaSuccess) { delete e; return MDGB_ERR_CUDA; }
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, c.device);
    if (!prop.cooperativeLaunch) { delete e; return MDGB_ERR_UNSUPPORTED; }
    e->num_sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) { delete e; return MDGB_ERR_CUDA; }
    int bps = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void*)k_pre, TILE, 0);
    int bps2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps2, (const void*)k_macro, TILE, 0);
    e->pre_blocks_per_sm = std::max(1, std::min(bps, bps2));
    if (list_build_init() != cudaSuccess) { cudaGetLastError(); delete e; return MDGB_ERR_CUDA; }
    lj_finish(e->pot_default);
    *out = e;
    return MDGB_OK;
}

MDGB_API int mdgb_destroy(mdgb_engine* e) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    delete e;
    return MDGB_OK;
}

MDGB_API const char* mdgb_last_error(const mdgb_engine* e) { return e ? e->err.c_str() : ""; }

MDGB_API const char* mdgb_status_string(int s) {
    switch (s) {
        case MDGB_OK: return "ok";
        case MDGB_ERR_INVALID_ARGUMENT: return "invalid argument";
        case MDGB_ERR_CUDA: return "CUDA error";
        case MDGB_ERR_NO_STATE: return "no state uploaded";
        case MDGB_ERR_NEIGHBOR_OVERFLOW: return "neighbour list overflow";
        case MDGB_ERR_FIXED_POINT_OVERFLOW: return "fixed-point force overflow";
        case MDGB_ERR_UNSUPPORTED: return "unsupported";
        case MDGB_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
        case MDGB_ERR_OUT_OF_MEMORY: return "out of device memory";
        case MDGB_ERR_SKIN_VIOLATION: return "skin violation";
        default: return "unknown status";
    }
}

MDGB_API void* mdgb_stream(mdgb_engine* e) { return e ? (void*)e->stream : nullptr; }

static int set_pot(mdgb_engine* e, uint16_t t0, uint16_t t1, const LJ& p) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    if (t0 >= MAX_TYPES || t1 >= MAX_TYPES) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "type id >= 16");
    const int a = std::min(t0, t1), b = std::max(t0, t1);  // potential.rs:142
    e->pot[a][b] = p;
    e->pot[a][b].set = true;
    if (e->has_state) {
        cudaSetDevice(e->device);
        int rc = upload_pairs(e);
        if (rc) return rc;
        e->graph_valid = false;
        // a changed cutoff needs lists built with the new radius
        CU(cudaMemcpyAsync(e->rep_host.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost,
                           e->stream));
        CU(cudaStreamSynchronize(e->stream));
        for (auto& R : e->rep_host) R.rebuild = 1;
        CU(cudaMemcpyAsync(e->dev.rep, e->rep_host.data(), e->nrep * sizeof(RepDev), cudaMemcpyHostToDevice,
                           e->stream));
    }
    return MDGB_OK;
}

MDGB_API int mdgb_set_potential(mdgb_engine* e, uint16_t t0, uint16_t t1, double sigma, double eps) {
    if (!(sigma > 0.0)) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "sigma must be positive");
    LJ p;
    p.sigma = sigma; p.eps = eps;
    lj_finish(p);
    return set_pot(e, t0, t1, p);
}

MDGB_API int mdgb_set_potential_raw(mdgb_engine* e, uint16_t t0, uint16_t t1, double sigma, double eps,
                                    double r_cut, double u_cut) {
    if (!(sigma > 0.0) || !(r_cut > 0.0)) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "bad potential");
    LJ p;
    p.sigma = sigma; p.eps = eps; p.rc = r_cut; p.ucut = u_cut;
    return set_pot(e, t0, t1, p);
}

MDGB_API int mdgb_upload_state(mdgb_engine* e, int64_t n, const uint16_t* type, const double* pos,
                               const double* vel, const double* mass_per_type, int ntypes, const double box[3]) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    const int64_t off[2] = {0, n};
    return upload_impl(e, 1, off, type, pos, vel, mass_per_type, ntypes, box);
}

MDGB_API int mdgb_ensemble_upload(mdgb_engine* e, int nrep, const int64_t* offsets, const uint16_t* type,
                                  const double* pos, const double* vel, const double* mass_per_type, int ntypes,
                                  const double* boxes) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return upload_impl(e, nrep, offsets, type, pos, vel, mass_per_type, ntypes, boxes);
}

MDGB_API int mdgb_upload_forces(mdgb_engine* e, const double* force, const double* potential,
                                const double* temp) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    cudaSetDevice(e->device);
    const size_t N = e->ntot;
    double* d_f = e->d_out;
    double* d_p = e->d_out + 3 * N;
    double* d_t = e->d_out + 4 * N;
    CU(cudaStreamSynchronize(e->stream));
    if (force) std::memcpy(e->h_pin, force, 3 * N * sizeof(double));
    if (potential) std::memcpy(e->h_pin + 3 * N, potential, N * sizeof(double));
    if (temp) std::memcpy(e->h_pin + 4 * N, temp, N * sizeof(double));
    CU(cudaMemcpyAsync(e->d_out, e->h_pin, 5 * N * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    const double* a = force ? d_f : nullptr;
    const double* b = potential ? d_p : nullptr;
    const double* c = temp ? d_t : nullptr;
    void* args[] = {(void*)&e->dev, (void*)&a, (void*)&b, (void*)&c};
    CU(cudaLaunchKernel((const void*)k_scatter_forces, dim3((unsigned)((N + 255) / 256)), dim3(256), args, 0,
                        e->stream));
    CU(cudaStreamSynchronize(e->stream));
    return MDGB_OK;
}

MDGB_API int mdgb_interacting_pairs(mdgb_engine* e, int64_t capacity, int32_t* out_i, int32_t* out_j,
                                    int64_t* count) {
    if (!e || !count || capacity < 0 || (capacity > 0 && (!out_i || !out_j))) return MDGB_ERR_INVALID_ARGUMENT;
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    cudaSetDevice(e->device);
    int* di = nullptr;
    int* dj = nullptr;
    unsigned long long* dc = nullptr;
    const size_t cap = (size_t)std::max<int64_t>(capacity, 1);
    CU(cudaMalloc(&di, cap * sizeof(int)));
    CU(cudaMalloc(&dj, cap * sizeof(int)));
    CU(cudaMalloc(&dc, sizeof(unsigned long long)));
    CU(cudaMemsetAsync(dc, 0, sizeof(unsigned long long), e->stream));
    long long lcap = capacity;
    void* args[] = {(void*)&e->dev, (void*)&lcap, (void*)&di, (void*)&dj, (void*)&dc};
    cudaError_t ce = cudaLaunchKernel((const void*)k_pairs, dim3((unsigned)((e->ntot + 127) / 128)), dim3(128), args,
                                      0, e->stream);
    unsigned long long total = 0;
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&total, dc, sizeof(total), cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    const size_t ncopy = (size_t)std::min<unsigned long long>(total, (unsigned long long)capacity);
    if (ce == cudaSuccess && ncopy) ce = cudaMemcpy(out_i, di, ncopy * sizeof(int), cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && ncopy) ce = cudaMemcpy(out_j, dj, ncopy * sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(di);
    cudaFree(dj);
    cudaFree(dc);
    if (ce != cudaSuccess) return fail(e, MDGB_ERR_CUDA, cudaGetErrorString(ce));
    *count = (int64_t)total;
    return MDGB_OK;
}

MDGB_API int mdgb_compute_forces(mdgb_engine* e) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    cudaSetDevice(e->device);
    if (!e->tuned) {
        int rc = autotune_tpa(e);
        if (rc) return rc;
    }
    int rc = compute_forces_impl(e);
    if (!rc) e->forces_valid = true;
    return rc;
}

MDGB_API int mdgb_step(mdgb_engine* e, int64_t nsteps, double dt, mdgb_thermostat* thermostat,
                       mdgb_barostat* barostat) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    if (e->nrep != 1) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "ensemble engine: use mdgb_ensemble_step");
    cudaSetDevice(e->device);
    int rc = set_coupling_impl(e, thermostat, barostat);
    if (rc) return rc;
    rc = step_impl(e, nsteps, dt);
    if (rc) return rc;
    return get_coupling_impl(e, thermostat, barostat);
}

MDGB_API int mdgb_download_state(mdgb_engine* e, double* pos, double* vel, double* force, double* potential,
                                 double* temp, double box[3]) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return download_impl(e, pos, vel, force, potential, temp, box);
}

MDGB_API int mdgb_macro_parameters(mdgb_engine* e, int type, mdgb_macro* out) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    if (e->nrep != 1) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "ensemble engine: use mdgb_ensemble_macro");
    cudaSetDevice(e->device);
    return macro_impl(e, type, out);
}

MDGB_API int mdgb_ensemble_set_coupling(mdgb_engine* e, const mdgb_thermostat* thermostats,
                                        const mdgb_barostat* barostats) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return set_coupling_impl(e, thermostats, barostats);
}

MDGB_API int mdgb_ensemble_step(mdgb_engine* e, int64_t nsteps, double dt) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return step_impl(e, nsteps, dt);
}

MDGB_API int mdgb_ensemble_get_coupling(mdgb_engine* e, mdgb_thermostat* thermostats, mdgb_barostat* barostats) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    cudaSetDevice(e->device);
    return get_coupling_impl(e, thermostats, barostats);
}

MDGB_API int mdgb_ensemble_download(mdgb_engine* e, double* pos, double* vel, double* force, double* potential,
                                    double* temp, double* boxes) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return download_impl(e, pos, vel, force, potential, temp, boxes);
}

MDGB_API int mdgb_ensemble_macro(mdgb_engine* e, int type, mdgb_macro* out) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return macro_impl(e, type, out);
}

MDGB_API int mdgb_get_stats(mdgb_engine* e, mdgb_stats* out) {
    if (!e || !out) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    prof_collect(e);
    if (e->has_state) {
        std::vector<RepDev> reps(e->nrep);
        if (cudaMemcpy(reps.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost) == cudaSuccess) {
            int64_t nb = 0;
            int mx = 0;
            for (auto& R : reps) { nb += R.nrebuilds; mx = std::max(mx, R.max_nn); }
            e->st.rebuilds = nb;
            e->st.max_neighbors = mx;
        }
    }
    e->st.neighbor_capacity = e->cap;
    e->st.threads_per_atom = e->tpa;
    for (int c = 0; c < mdgb_engine::NCLASS; ++c) {
        e->st.class_threads_per_atom[c] = e->class_tpa[c];
        e->st.class_replicas[c] = e->class_nrep[c];
    }
    *out = e->st;
    return MDGB_OK;
}

MDGB_API int mdgb_trace_phases(mdgb_engine* e, double* out, int n) {
    if (!e || !out || n < 0) return MDGB_ERR_INVALID_ARGUMENT;
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    if (!(e->cfg.flags & MDGB_FLAG_TRACE)) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "engine created without MDGB_FLAG_TRACE");
    cudaSetDevice(e->device);
    unsigned long long h[TR_SLOTS];
    CU(cudaMemcpyAsync(h, e->trace_buf, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    CU(cudaMemsetAsync(e->trace_buf, 0, sizeof(h), e->stream));
    const int m = std::min(n, 14);
    for (int i = 0; i < m; ++i) out[i] = i < 12 ? h[i] * 1e-3 : (double)h[i];
    return MDGB_OK;
}

MDGB_API int mdgb_reset_stats(mdgb_engine* e) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    prof_collect(e);
    const int cap = e->st.neighbor_capacity;
    e->st = mdgb_stats{};
    e->st.neighbor_capacity = cap;
    if (e->has_state) {
        std::vector<RepDev> reps(e->nrep);
        if (cudaMemcpy(reps.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost) == cudaSuccess) {
            for (auto& R : reps) R.nrebuilds = 0;
            cudaMemcpy(e->dev.rep, reps.data(), e->nrep * sizeof(RepDev), cudaMemcpyHostToDevice);
        }
    }
    return MDGB_OK;
}

MDGB_API int mdgb_synchronize(mdgb_engine* e) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return cudaStreamSynchronize(e->stream) == cudaSuccess ? MDGB_OK : MDGB_ERR_CUDA;
}

}  // extern "C"
