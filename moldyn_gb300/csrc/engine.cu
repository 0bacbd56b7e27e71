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
__global__ void k_scatter_in(Dev d, const double*, const double*, const uint16_t*, const int*, int);
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
    // the force launches of the size classes after the first run on their own
    // streams, forked from and joined back into `stream` (also inside graphs)
    cudaStream_t aux[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[3] = {nullptr, nullptr, nullptr};
    int num_sms = 0;
    // the GPU reads the caller's pageable arrays itself (Grace: address
    // translation through the host's page tables), so uploads skip the copy
    bool host_direct = false;
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
    // Verlet skin of each size class (a replica's list radius is the largest
    // r_cut plus its class's skin): the configured skin, or tuned on the
    // first step call when the configuration leaves it to the engine
    double class_skin[NCLASS] = {0.0, 0.0, 0.0};
    bool skin_tuned = false;

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
    // device staging in the caller's order; host arrays are copied to and
    // from it directly (no pinned host copy: on this platform the copy engine
    // reads and writes pageable memory at full link speed)
    double* d_out = nullptr;     // [11][N] caller-order staging (pos, vel, force, potential, temp)
    int* d_in_i = nullptr;       // [N] reference ranks (several types)
    uint16_t* d_in_t = nullptr;  // [N] caller type ids
    int* h_err = nullptr;        // pinned
    unsigned long long* trace_buf = nullptr;  // per-phase ns of k_pre (MDGB_FLAG_TRACE)
    int lb_grid = 1, lm_grid = 1, lb_cap = -1, lb_ncells = -1;  // list-build launch shapes for (cap, cells)
    // the other position / mirror buffer of each pair (fused NVE drift)
    double4_32a* pos_alt = nullptr;
    float4* mir_alt = nullptr;
    // coupling (host view of the per-replica settings)
    bool thermo_on = false, baro_on = false, thermo_nh = false;

    // captured step chunks: one graph per distinct chunk length and launch
    // parameters (the key holds everything a capture bakes in), replayed
    // whenever a chunk with the same key comes again; a few are kept
    struct GraphKey {
        int len, lb_grid;
        unsigned flags;
        int precision;
        StepParams sp;
        Dev dev;
        const void* pos_alt;
        const void* mir_alt;
        int class_tpa[3], class_ntiles[3], class_tile_off[3], lm_grid;
    };
    struct GraphEntry {
        GraphKey key;
        cudaGraphExec_t exec;
        int64_t kernels;         // kernel launches one replay makes
        uint64_t used;
    };
    std::vector<GraphEntry> graphs;
    uint64_t graph_clock = 0;
    // the cells and lists were built at the current positions and nothing has
    // moved since (a force evaluation can skip its rebuild)
    bool lists_fresh = false;
    // failure test of the bounded grid barrier (mdgb_test_barrier_timeout):
    // the next step call's first chunk holds this block back (-1: off)
    int test_hold_block = -1;
    long long test_barrier_cycles = 0;

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

void drop_graphs(mdgb_engine* e) {
    for (auto& g : e->graphs) cudaGraphExecDestroy(g.exec);
    e->graphs.clear();
}

// Device allocations of a state (kept by an upload of the same shape).
void free_state(mdgb_engine* e) {
    drop_graphs(e);
    for (void* p : e->allocs) cudaFree(p);
    e->allocs.clear();
    if (e->nbr_alloc) { cudaFree(e->nbr_alloc); e->nbr_alloc = nullptr; }
    e->dev.nn = nullptr;
    e->has_state = false;
    e->forces_valid = false;
    e->lists_fresh = false;
}

const LJ& pot_of(const mdgb_engine* e, int a, int b) {
    if (a > b) std::swap(a, b);
    return e->pot[a][b].set ? e->pot[a][b] : e->pot_default;
}

// Skin of size class c: the tuned one, else the configured (or default) one.
double class_skin_of(const mdgb_engine* e, int c) { return e->skin_tuned ? e->class_skin[c] : e->skin; }

// The configuration asks the engine to choose the skin (skin < 0; 0 means
// the default skin).  The choice comes from timings, and on the mixed path
// the cell grid it implies changes FP32 roundings, so tuning is opt-in: an
// untuned run is reproducible bit for bit.  Reference-order runs keep the
// default (their sums do not depend on the list).
bool skin_auto(const mdgb_engine* e) {
    return e->cfg.skin < 0.0 && !((e->cfg.flags & MDGB_FLAG_REFERENCE_ORDER) && e->cfg.precision == MDGB_PRECISION_FP64);
}

// Skin candidates of the tuning, as fractions of the largest r_cut
// (0.2 .. 0.4 sigma at r_cut = 2.5 sigma).
constexpr double SKIN_FRACTIONS[5] = {0.08, 0.10, 0.12, 0.14, 0.16};

// The largest list radius of any replica (the force kernels' range bounds).
void update_rlist(mdgb_engine* e) {
    double smax = e->skin;
    for (int c = 0; c < mdgb_engine::NCLASS; ++c)
        if (e->class_ntiles[c]) smax = std::max(smax, class_skin_of(e, c));
    e->rlist = e->rcmax + smax;
    e->dev.rlist = e->rlist;
}

// The pair table of the current potentials and the scalars derived from it
// (largest cut-off, list radius, fixed-point scale), on the host.
std::vector<PairDev> pair_table(mdgb_engine* e) {
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
    // fixed-point scale: a power of two putting the characteristic force near 2^31
    if (!(fchar > 0.0)) fchar = 1.0;
    const int ex = 31 - (int)std::ceil(std::log2(fchar));
    e->dev.fscale = std::ldexp(1.0f, ex);
    e->dev.fscale_log2 = ex;
    e->dev.inv_fscale = std::ldexp(1.0, -ex);
    e->dev.inv_fscale_f = std::ldexp(1.0f, -ex);
    e->skin = e->cfg.skin > 0.0 ? e->cfg.skin : 0.12 * e->rcmax;
    update_rlist(e);
    e->dev.rcmax = e->rcmax;
    e->dev.skin = e->skin;
    return tab;
}

int upload_pairs(mdgb_engine* e) {
    const std::vector<PairDev> tab = pair_table(e);
    CU(cudaMemcpyAsync((void*)e->dev.pair, tab.data(), tab.size() * sizeof(PairDev),
                       cudaMemcpyHostToDevice, e->stream));
    CU(cudaStreamSynchronize(e->stream));   // the table is a local copy
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
    e->lists_fresh = false;
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
        e->lm_grid = list_masks_grid(e->dev, e->num_sms);
        e->lb_cap = e->dev.cap;
        e->lb_ncells = e->dev.ncells;
    }
    CU(launch_list_build(e->dev, e->lb_grid, e->lm_grid, e->stream));
    prof_end(e, pe);
    e->st.kernel_launches += 3;
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
int launch_force_class(mdgb_engine* e, const StepParams& sp, bool kick, int c, cudaStream_t st) {
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
    CU(cudaLaunchKernel((const void*)fn, dim3(grid), dim3(TILE * tpa), args, 0, st));
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
    // classes touch disjoint atoms, tiles and queue counters: the second and
    // third run concurrently with the first on their own streams
    int nclasses = 0;
    for (int c = 0; c < mdgb_engine::NCLASS; ++c) nclasses += e->class_ntiles[c] ? 1 : 0;
    bool first = true;
    for (int c = 0; c < mdgb_engine::NCLASS; ++c) {
        if (!e->class_ntiles[c]) continue;
        int rc;
        if (first) {
            if (nclasses > 1) CU(cudaEventRecord(e->fork_ev, e->stream));
            rc = launch_force_class(e, sp, kick, c, e->stream);
            first = false;
        } else {
            CU(cudaStreamWaitEvent(e->aux[c], e->fork_ev, 0));
            rc = launch_force_class(e, sp, kick, c, e->aux[c]);
            if (!rc) CU(cudaEventRecord(e->join_ev[c], e->aux[c]));
            if (!rc) CU(cudaStreamWaitEvent(e->stream, e->join_ev[c], 0));
        }
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
    bool changed = false;
    for (int r = 0; r < e->nrep; ++r) {
        const int t = e->class_tpa[e->class_of[r]];
        changed |= e->rep_host[r].tpa != t;
        e->rep_host[r].tpa = t;
    }
    if (!changed) return MDGB_OK;
    CU(cudaMemcpyAsync(e->dev.rep, e->rep_host.data(), e->nrep * sizeof(RepDev), cudaMemcpyHostToDevice, e->stream));
    e->lists_fresh = false;   // the list layout changed
    return MDGB_OK;
}

// Each replica's list radius: the largest r_cut plus its size class's skin.
int apply_class_skin(mdgb_engine* e) {
    CU(cudaMemcpyAsync(e->rep_host.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    for (int r = 0; r < e->nrep; ++r) e->rep_host[r].rlist = e->rcmax + class_skin_of(e, e->class_of[r]);
    CU(cudaMemcpyAsync(e->dev.rep, e->rep_host.data(), e->nrep * sizeof(RepDev), cudaMemcpyHostToDevice, e->stream));
    update_rlist(e);
    e->lists_fresh = false;
    return MDGB_OK;
}

StepParams make_sp(const mdgb_engine* e, double dt, bool drift) {
    StepParams sp;
    std::memset(&sp, 0, sizeof(sp));   // byte-wise comparable (graph keys)
    sp.hold_block = -1;
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
    // bar[5] (direct list builds) is a counter: kept
    CU(cudaMemsetAsync(e->dev.bar, 0, 5 * sizeof(unsigned int), e->stream));
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
    if (flags & E_INPUT) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "type id >= ntypes");
    if (flags & (E_BOUNDS | E_CELLS)) return fail(e, MDGB_ERR_CUDA, "internal index check failed");
    return MDGB_OK;
}

// Forced rebuild of cells and lists at the current positions; a list that
// overflows is grown and built again.
int rebuild_lists(mdgb_engine* e) {
    for (int attempt = 0; attempt < 8; ++attempt) {
        int rc = clear_err(e);
        if (rc) return rc;
        rc = refresh(e, true);
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
        rc = check_flags(e, flags);
        if (rc) return rc;
        e->lists_fresh = true;
        return MDGB_OK;
    }
    return fail(e, MDGB_ERR_NEIGHBOR_OVERFLOW, "neighbour list kept overflowing");
}

// update_force: a rebuild (skipped when the lists were just built at these
// positions -- a second one would give the same cells and lists), then the
// force pass.
int compute_forces_impl(mdgb_engine* e) {
    for (int attempt = 0; attempt < 8; ++attempt) {
        int rc = clear_err(e);
        if (rc) return rc;
        if (!e->lists_fresh) {
            rc = refresh(e, true);
            if (rc) return rc;
        }
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
        rc = check_flags(e, flags);
        if (rc) return rc;
        e->lists_fresh = true;
        return MDGB_OK;
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

mdgb_engine::GraphKey graph_key(const mdgb_engine* e, const StepParams& sp, int n) {
    mdgb_engine::GraphKey k;
    std::memset(&k, 0, sizeof(k));   // padding included: keys compare as bytes
    k.len = n;
    k.lb_grid = e->lb_grid;
    k.lm_grid = e->lm_grid;
    k.flags = e->cfg.flags;
    k.precision = e->cfg.precision;
    k.sp = sp;
    k.dev = e->dev;
    k.pos_alt = e->pos_alt;
    k.mir_alt = e->mir_alt;
    for (int c = 0; c < mdgb_engine::NCLASS; ++c) {
        k.class_tpa[c] = e->class_tpa[c];
        k.class_ntiles[c] = e->class_ntiles[c];
        k.class_tile_off[c] = e->class_tile_off[c];
    }
    return k;
}

// The graph of a chunk of n steps with these parameters, captured on first
// use (capture runs nothing).  Returns null when graphs are off or capture is
// not possible here (the engine then stays eager).
mdgb_engine::GraphEntry* chunk_graph(mdgb_engine* e, const StepParams& sp, int n, int* rc_out) {
    *rc_out = MDGB_OK;
    if (!(e->cfg.graph_steps > 1) || (e->cfg.flags & MDGB_FLAG_PROFILE)) return nullptr;
    // the list-build grid is part of the key: settle it before the lookup
    if (e->lb_cap != e->dev.cap || e->lb_ncells != e->dev.ncells) {
        e->lb_grid = list_build_grid(e->dev, e->num_sms);
        e->lm_grid = list_masks_grid(e->dev, e->num_sms);
        e->lb_cap = e->dev.cap;
        e->lb_ncells = e->dev.ncells;
    }
    const mdgb_engine::GraphKey key = graph_key(e, sp, n);
    for (auto& g : e->graphs)
        if (std::memcmp(&g.key, &key, sizeof(key)) == 0) {
            g.used = ++e->graph_clock;
            return &g;
        }
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal);
    if (ce != cudaSuccess) { *rc_out = fail(e, MDGB_ERR_CUDA, cudaGetErrorString(ce)); return nullptr; }
    const int64_t launches0 = e->st.kernel_launches;
    // capture runs nothing: the buffer pair must read as before afterwards
    double4_32a* const pos0 = e->dev.pos; double4_32a* const pos1 = e->pos_alt;
    float4* const mir0 = e->dev.mir; float4* const mir1 = e->mir_alt;
    int rc = run_chunk_kernels(e, sp, n);
    ce = cudaStreamEndCapture(e->stream, &g);
    e->dev.pos = pos0; e->pos_alt = pos1; e->dev.mir = mir0; e->mir_alt = mir1;
    const int64_t kernels = e->st.kernel_launches - launches0;
    e->st.kernel_launches = launches0;
    cudaGraphExec_t exec = nullptr;
    if (!rc && ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (rc || ce != cudaSuccess) {
        cudaGetLastError();
        e->cfg.graph_steps = 0;  // capture unsupported here: stay eager
        return nullptr;
    }
    if (e->graphs.size() >= 6) {   // drop the least recently used
        size_t lru = 0;
        for (size_t i = 1; i < e->graphs.size(); ++i)
            if (e->graphs[i].used < e->graphs[lru].used) lru = i;
        cudaGraphExecDestroy(e->graphs[lru].exec);
        e->graphs.erase(e->graphs.begin() + (long)lru);
    }
    e->graphs.push_back(mdgb_engine::GraphEntry{key, exec, kernels, ++e->graph_clock});
    return &e->graphs.back();
}

int run_chunk(mdgb_engine* e, const StepParams& sp, int n) {
    int rc = MDGB_OK;
    mdgb_engine::GraphEntry* g = chunk_graph(e, sp, n, &rc);
    if (rc) return rc;
    if (!g) return run_chunk_kernels(e, sp, n);
    CU(cudaGraphLaunch(g->exec, e->stream));
    e->st.graph_launches++;
    e->st.kernel_launches += g->kernels;
    return MDGB_OK;
}

// Chunk lengths a call of nsteps steps runs: full chunks, then the rest.
int chunk_steps(const mdgb_engine* e) { return e->cfg.graph_steps > 1 ? e->cfg.graph_steps : 64; }

int autotune_tpa(mdgb_engine* e);
int autotune_skin(mdgb_engine* e, double dt);

int step_impl(mdgb_engine* e, int64_t nsteps, double dt) {
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    if (nsteps < 0 || !(dt == dt)) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "bad nsteps or dt");
    if (!e->tuned) {
        int rc = autotune_tpa(e);
        if (rc) return rc;
    }
    if (nsteps > 0 && !e->skin_tuned && skin_auto(e)) {
        int rc = autotune_skin(e, dt);
        if (rc) return rc;
    }
    const StepParams sp = make_sp(e, dt, true);
    const int chunk = chunk_steps(e);
    if (nsteps > 0) e->lists_fresh = false;
    int64_t done = 0;
    int retries = 0;
    while (done < nsteps) {
        const int n = (int)std::min<int64_t>(chunk, nsteps - done);
        int rc = clear_err(e);
        if (rc) return rc;
        rc = snapshot(e, false);
        if (rc) return rc;
        if (e->test_hold_block >= 0) {
            // the armed failure test: this chunk eager, its first step kernel
            // with one block held back and a short wait limit
            StepParams t = sp;
            t.hold_block = e->test_hold_block;
            t.barrier_cycles = e->test_barrier_cycles;
            e->test_hold_block = -1;
            rc = run_chunk_kernels(e, t, n);
        } else {
            rc = run_chunk(e, sp, n);
        }
        if (rc) return rc;
        int flags = 0;
        rc = read_err(e, &flags);
        if (rc) return rc;
        if (flags & E_TIMEOUT) {
            // a grid barrier gave up: the rest of the chunk did nothing; put
            // the state back as the chunk found it, so the engine stays usable
            rc = snapshot(e, true);
            if (!rc) rc = rebuild_lists(e);
            if (rc) return rc;
            return fail(e, MDGB_ERR_DEVICE_TIMEOUT,
                        "a device-side grid barrier timed out; the state is as before the failed chunk");
        }
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

// Capture, without running anything, the graphs a call of nsteps steps with
// these coupling kinds will replay (the full chunk and the remainder), so the
// first such call does not pay for the capture.
int prepare_impl(mdgb_engine* e, int64_t nsteps, double dt, bool thermo_on, bool baro_on, bool thermo_nh) {
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    if (nsteps < 0 || !(dt == dt)) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "bad nsteps or dt");
    if (!(e->cfg.graph_steps > 1)) return MDGB_OK;   // eager engine: nothing to capture
    if (!e->tuned) {
        int rc = autotune_tpa(e);
        if (rc) return rc;
    }
    const bool t0 = e->thermo_on, b0 = e->baro_on, n0 = e->thermo_nh;
    if (nsteps > 0 && !e->skin_tuned && skin_auto(e)) {
        // the tuning runs steps: with the coupling kinds of the later call
        e->thermo_on = thermo_on; e->baro_on = baro_on; e->thermo_nh = thermo_nh;
        const int rc = autotune_skin(e, dt);
        e->thermo_on = t0; e->baro_on = b0; e->thermo_nh = n0;
        if (rc) return rc;
    }
    e->thermo_on = thermo_on; e->baro_on = baro_on; e->thermo_nh = thermo_nh;
    const StepParams sp = make_sp(e, dt, true);
    e->thermo_on = t0; e->baro_on = b0; e->thermo_nh = n0;
    const int chunk = chunk_steps(e);
    const int64_t lens[2] = {std::min<int64_t>(chunk, nsteps), nsteps > chunk ? nsteps % chunk : 0};
    for (int64_t len : lens) {
        if (len <= 0) continue;
        int rc = MDGB_OK;
        chunk_graph(e, sp, (int)len, &rc);
        if (rc) return rc;
    }
    return MDGB_OK;
}

// Skin of each size class, for the step's own dynamics: from the state the
// first step call starts from, each candidate (SKIN_FRACTIONS of the largest
// r_cut) runs a short stretch of steps (eager launches, CUDA-event timed, its
// rebuilds included) and the state is put back; classes are tuned one after
// the other, each keeping its fastest.  A larger skin means longer lists but
// fewer rebuilds.  The steps taken here are not counted and leave no trace:
// the state afterwards is the one the call started from.
int autotune_skin(mdgb_engine* e, double dt) {
    constexpr int NC = mdgb_engine::NCLASS;
    constexpr int K = 40;
    for (int c = 0; c < NC; ++c) e->class_skin[c] = e->skin;
    e->skin_tuned = true;   // class_skin now holds the values in use
    const unsigned saved_flags = e->cfg.flags;
    const int64_t launches0 = e->st.kernel_launches;
    e->cfg.flags &= ~MDGB_FLAG_PROFILE;
    const StepParams sp = make_sp(e, dt, true);
    int rc = snapshot(e, false);   // the state the call started from
    unsigned long long trace0[TR_SLOTS];   // the tuning's steps stay out of the phase trace
    if (!rc) {
        CU(cudaMemcpyAsync(trace0, e->trace_buf, sizeof(trace0), cudaMemcpyDeviceToHost, e->stream));
        CU(cudaStreamSynchronize(e->stream));
    }
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (!rc && (cudaEventCreate(&ev[0]) != cudaSuccess || cudaEventCreate(&ev[1]) != cudaSuccess))
        rc = fail(e, MDGB_ERR_CUDA, "cudaEventCreate failed");
    for (int c = 0; c < NC && !rc; ++c) {
        if (!e->class_ntiles[c]) continue;
        float best = 1e30f;
        double best_skin = e->class_skin[c];
        for (int k = 0; k < 5 && !rc; ++k) {
            e->class_skin[c] = SKIN_FRACTIONS[k] * e->rcmax;
            bool done = false;
            for (int attempt = 0; attempt < 8 && !done && !rc; ++attempt) {
                rc = snapshot(e, true);
                if (!rc) rc = apply_class_skin(e);
                if (!rc) rc = rebuild_lists(e);
                if (!rc) rc = clear_err(e);
                if (rc) break;
                if (cudaEventRecord(ev[0], e->stream) != cudaSuccess) { rc = fail(e, MDGB_ERR_CUDA, "event"); break; }
                rc = run_chunk_kernels(e, sp, K);
                if (rc) break;
                if (cudaEventRecord(ev[1], e->stream) != cudaSuccess) { rc = fail(e, MDGB_ERR_CUDA, "event"); break; }
                int flags = 0;
                rc = read_err(e, &flags);
                if (rc) break;
                if (flags & E_NLIST) {   // longer lists: grow and time this candidate again
                    rc = grow_list(e);
                    continue;
                }
                rc = check_flags(e, flags);
                if (rc) break;
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, ev[0], ev[1]) != cudaSuccess) { rc = fail(e, MDGB_ERR_CUDA, "event"); break; }
                if (ms < best) { best = ms; best_skin = e->class_skin[c]; }
                done = true;
            }
        }
        e->class_skin[c] = best_skin;
    }
    for (auto& x : ev)
        if (x) cudaEventDestroy(x);
    e->cfg.flags = saved_flags;
    e->st.kernel_launches = launches0;
    if (rc) return rc;
    // back to the starting state; its lists are rebuilt with the chosen skins
    // (a real rebuild, counted and traced like any other)
    CU(cudaMemcpyAsync(e->trace_buf, trace0, sizeof(trace0), cudaMemcpyHostToDevice, e->stream));
    rc = snapshot(e, true);
    if (!rc) rc = apply_class_skin(e);
    if (!rc) rc = rebuild_lists(e);
    return rc;
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
        return e->lists_fresh ? MDGB_OK : rebuild_lists(e);
    }
    e->lists_fresh = false;
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
            for (int i = 0; i < 3 && !rc; ++i) rc = launch_force_class(e, sp, false, c, e->stream);
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
    if (rc) return rc;
    return rebuild_lists(e);  // lists in the chosen layouts
}

// Upload of a state (one replica or an ensemble).  An upload whose shape
// (atoms, replicas, tiles, cells, reduction chunks) equals the previous one
// keeps the device allocations, the neighbour list (if large enough), the
// tuned threads per atom and the captured graphs; anything else starts over.
// The caller's arrays are copied straight to the device (pageable memory is
// fine) and scattered into the device layout by a kernel.
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
            if (!(boxes[3 * r + a] > 0.0) || !std::isfinite(boxes[3 * r + a]))
                return fail(e, MDGB_ERR_INVALID_ARGUMENT, "box must be positive and finite");
    }
    for (int t = 0; t < ntypes; ++t)
        if (!(mass_per_type[t] > 0.0)) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "mass must be positive");
    const int N = (int)n;

    // reference ranks (type-major within each replica) and per-replica type
    // offsets; with one type the rank is the index itself and the type ids are
    // checked on the device
    std::vector<int> rank;
    std::vector<RepDev> reps(nrep, RepDev{});
    if (ntypes > 1) {
        rank.resize(N);
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
            RepDev& R = reps[r];
            for (int t = 0; t <= ntypes; ++t) R.type_off[t] = (int)cnt[t];
            for (int t = ntypes + 1; t <= MAX_TYPES; ++t) R.type_off[t] = (int)cnt[ntypes];
            std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
            for (int64_t i = offsets[r]; i < offsets[r + 1]; ++i) rank[i] = (int)(offsets[r] + fill[type[i]]++);
            R.last_type_count = (int)(cnt[ntypes] - cnt[ntypes - 1]);
        }
    } else {
        for (int r = 0; r < nrep; ++r) {
            RepDev& R = reps[r];
            const int nr = (int)(offsets[r + 1] - offsets[r]);
            R.type_off[0] = 0;
            for (int t = 1; t <= MAX_TYPES; ++t) R.type_off[t] = nr;
            R.last_type_count = nr;
        }
    }

    // potentials and list radius (host side: the cell capacity depends on it)
    e->ntypes = ntypes;
    e->dev.ntypes = ntypes;
    const std::vector<PairDev> pair_tab = pair_table(e);

    // tiles and cells (cell capacity for the smallest list radius the skin
    // tuning may choose)
    const bool auto_skin = skin_auto(e);
    const double rl_cells = e->rcmax + (auto_skin ? std::min(e->skin, SKIN_FRACTIONS[0] * e->rcmax) : e->skin);
    std::vector<int4> tiles;
    std::vector<int> cell_rep;
    int max_rep_n = 0;
    double max_density = 0.0;
    for (int r = 0; r < nrep; ++r) {
        RepDev& R = reps[r];
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
            prod *= std::max(1.0, std::floor(L / (rl_cells * (1.0 + 1e-6))));
        }
        const double vol = boxes[3 * r] * boxes[3 * r + 1] * boxes[3 * r + 2];
        max_density = std::max(max_density, nr / vol);
        // cell capacity: the grid at this box with room to grow (barostat), but
        // no finer than ~8 atoms a cell -- a dilute replica gets larger
        // cells, so its rebuild is not dominated by per-cell work
        const double capd = std::min(std::ceil(prod * 1.3) + 27.0, nr / 8.0 + 27.0);
        R.cell_cap = (int)std::max(27.0, capd);
        R.cell_base = (int)cell_rep.size();
        cell_rep.insert(cell_rep.end(), R.cell_cap, r);
        R.mode = MODE_BRUTE;
        R.pending = 1.0;
        R.lambda = 0.0;
        R.myu = 0.0;
        R.rebuild = 1;
    }
    const int ntiles = (int)tiles.size();
    const int ncells = (int)cell_rep.size();
    // reduction chunks: runs of <= CHUNK_TILES tiles inside one replica
    std::vector<int4> chunks;
    for (int r = 0; r < nrep; ++r) {
        RepDev& R = reps[r];
        R.chunk_begin = (int)chunks.size();
        for (int t = 0; t < R.ntiles; t += CHUNK_TILES)
            chunks.push_back(make_int4(r, R.tile_begin + t, std::min(CHUNK_TILES, R.ntiles - t), 0));
        R.nchunks = (int)chunks.size() - R.chunk_begin;
    }

    // size classes by replica atom count; tile_order = class 0 tiles, class 1, class 2,
    // costliest (densest replica) first inside a class (persistent kernel)
    constexpr int NC = mdgb_engine::NCLASS;
    std::vector<int> class_of(nrep, 0);
    int class_ntiles[NC] = {0, 0, 0}, class_nrep[NC] = {0, 0, 0};
    for (int r = 0; r < nrep; ++r) {
        const int nr = reps[r].n;
        const int c = nr < 2048 ? 0 : (nr < 32768 ? 1 : 2);
        class_of[r] = c;
        reps[r].size_class = c;
        class_nrep[c]++;
        class_ntiles[c] += reps[r].ntiles;
    }
    std::vector<int> order(ntiles);
    for (int i = 0; i < ntiles; ++i) order[i] = i;
    if (nrep > 1) {
        // expected pair work of a tile: its atoms x the replica's neighbours per atom
        const double sphere = 4.0 / 3.0 * M_PI * e->rlist * e->rlist * e->rlist;
        std::vector<double> rep_cost(nrep);
        for (int r = 0; r < nrep; ++r) {
            const RepDev& R = reps[r];
            const double dens = R.n / (R.box[0] * R.box[1] * R.box[2]);
            rep_cost[r] = std::min((double)R.n, 1.0 + dens * sphere);
        }
        struct Key { int cls; double cost; int tile; };
        std::vector<Key> key(ntiles);
        for (int i = 0; i < ntiles; ++i) key[i] = {class_of[tiles[i].x], tiles[i].z * rep_cost[tiles[i].x], i};
        std::stable_sort(key.begin(), key.end(), [](const Key& a, const Key& b) {
            return a.cls != b.cls ? a.cls < b.cls : a.cost > b.cost;
        });
        for (int i = 0; i < ntiles; ++i) order[i] = key[i].tile;
    }

    // keep the allocations when the shape is unchanged
    Dev& d = e->dev;
    const bool reuse = e->has_state && N == e->ntot && nrep == e->nrep && ntiles == e->ntiles &&
                       ncells == e->ncells && (int)chunks.size() == d.nchunks;
    bool same_classes = reuse;
    for (int c = 0; c < NC; ++c)
        same_classes = same_classes && class_ntiles[c] == e->class_ntiles[c] && class_nrep[c] == e->class_nrep[c];
    if (!reuse) free_state(e);
    if (!same_classes) e->skin_tuned = false;
    e->has_state = false;
    e->forces_valid = false;
    e->lists_fresh = false;
    e->ntot = N;
    e->nrep = nrep;
    e->ntiles = ntiles;
    e->ncells = ncells;
    e->offsets.assign(offsets, offsets + nrep + 1);
    e->mass.assign(mass_per_type, mass_per_type + ntypes);
    e->rep_host = reps;
    e->class_of = class_of;
    for (int c = 0; c < NC; ++c) { e->class_ntiles[c] = class_ntiles[c]; e->class_nrep[c] = class_nrep[c]; }
    e->class_tile_off[0] = 0;
    for (int c = 1; c < NC; ++c) e->class_tile_off[c] = e->class_tile_off[c - 1] + e->class_ntiles[c - 1];

    d.ntot = N; d.ntiles = ntiles; d.nrep = nrep; d.ncells = ncells;
    d.refmode = (e->cfg.flags & MDGB_FLAG_REFERENCE_ORDER) && e->cfg.precision == MDGB_PRECISION_FP64 ? 1 : 0;
    d.mixed = e->cfg.precision != MDGB_PRECISION_FP64 ? 1 : 0;
    d.single_type = ntypes == 1 ? 1 : 0;
    d.direct_list = (e->cfg.flags & MDGB_FLAG_DIRECT_LIST) ? 1 : 0;
    d.last_type = ntypes - 1;
    for (int t = 0; t < MAX_TYPES; ++t) d.mass[t] = t < ntypes ? mass_per_type[t] : 1.0;

    int rc = MDGB_OK;
    if (!reuse) {
        if ((rc = dalloc(e, (PairDev**)&d.pair, MAX_TYPES * MAX_TYPES)) ||
            (rc = dalloc(e, &d.pos, N)) || (rc = dalloc(e, &d.vel, 3 * (size_t)N)) ||
            (rc = dalloc(e, &d.frc, 3 * (size_t)N)) || (rc = dalloc(e, &d.epot, N)) ||
            (rc = dalloc(e, &d.evir, N)) || (rc = dalloc(e, &d.mir, N)) || (rc = dalloc(e, &d.mir0, N)) ||
            (rc = dalloc(e, &e->pos_alt, N)) || (rc = dalloc(e, &e->mir_alt, N)) ||
            (rc = dalloc(e, &d.band_list, N)) || (rc = dalloc(e, &d.band_count, 1)) ||
            (rc = dalloc(e, &d.cell, N)) || (rc = dalloc(e, &d.orig, N)) || (rc = dalloc(e, &d.rank, N)) ||
            (rc = dalloc(e, &d.nn, N)) || (rc = dalloc(e, &d.tiles, ntiles)) ||
            (rc = dalloc(e, &d.rep, nrep)) || (rc = dalloc(e, &d.part, 8 * (size_t)ntiles)) ||
            (rc = dalloc(e, &d.cpart, 8 * chunks.size())) || (rc = dalloc(e, &d.chunks, chunks.size())) ||
            (rc = dalloc(e, &d.fx_part, ntiles)) || (rc = dalloc(e, &d.fx_cpart, chunks.size())) ||
            (rc = dalloc(e, &d.err, 2)) || (rc = dalloc(e, &d.max_needed, 1)) ||
            (rc = dalloc(e, &d.cell_count, ncells)) ||
            (rc = dalloc(e, &d.cell_start, ncells + 1)) || (rc = dalloc(e, &d.cell_rep, ncells)) ||
            (rc = dalloc(e, &d.perm, N)) || (rc = dalloc(e, &d.tmp_pos, N)) ||
            (rc = dalloc(e, &d.tmp_d, 8 * (size_t)N)) || (rc = dalloc(e, &d.tmp_i, 4 * (size_t)N)) ||
            (rc = dalloc(e, &d.slot_of_rank, N)) || (rc = dalloc(e, &d.bsum, 4096)) ||
            (rc = dalloc(e, &d.lmask, 27 * (size_t)N)) || (rc = dalloc(e, &d.nbs, 27 * (size_t)ncells)) ||
            (rc = dalloc(e, &d.rb, 4 + 3 * (size_t)nrep)) ||
            (rc = dalloc(e, &d.bar, 8)) || (rc = dalloc(e, &d.queue, NC)) ||
            (rc = dalloc(e, &e->trace_buf, TR_SLOTS)) ||
            (rc = dalloc(e, &d.tile_order, ntiles)) ||
            (rc = dalloc(e, &e->snap_pos, N)) || (rc = dalloc(e, &e->snap_d, 8 * (size_t)N)) ||
            (rc = dalloc(e, &e->snap_i, 4 * (size_t)N)) || (rc = dalloc(e, &e->snap_mir0, N)) ||
            (rc = dalloc(e, &e->snap_rep, nrep)) || (rc = dalloc(e, &e->d_out, 11 * (size_t)N)) ||
            (rc = dalloc(e, &e->d_in_i, N)) || (rc = dalloc(e, &e->d_in_t, N)))
            return rc;
    }
    if (!e->h_err) CU(cudaMallocHost((void**)&e->h_err, 4 * sizeof(int)));
    CU(cudaMemcpyAsync((void*)d.pair, pair_tab.data(), pair_tab.size() * sizeof(PairDev), cudaMemcpyHostToDevice,
                       e->stream));

    // neighbour capacity from the densest replica (grows on overflow)
    int cap = e->cfg.neighbor_capacity;
    if (cap <= 0) {
        const double expect = 4.0 / 3.0 * M_PI * std::pow(e->rlist * (1.0 + 1e-5), 3) * max_density;
        cap = (int)std::ceil(expect * 1.35 + 16.0);
        cap = std::min(cap, std::max(max_rep_n - 1, 8));
    }
    cap = std::max(8, (cap + 7) & ~7);
    if (!e->nbr_alloc || cap > e->cap) {
        rc = alloc_nbr(e, cap);
        if (rc) return rc;
    }
    e->st = mdgb_stats{};
    e->st.neighbor_capacity = e->cap;

    // threads per atom: kept from the last tuning when the size classes are
    // the same, else the configured (or default) value until the next tuning
    if (!same_classes) {
        const int t0 = d.refmode ? 1 : (e->cfg.threads_per_atom > 0 ? e->cfg.threads_per_atom : 1);
        for (int c = 0; c < NC; ++c) e->class_tpa[c] = t0;
        e->tuned = false;
    }
    for (int r = 0; r < nrep; ++r) {
        e->rep_host[r].tpa = e->class_tpa[e->class_of[r]];
        e->rep_host[r].rlist = e->rcmax + class_skin_of(e, e->class_of[r]);
    }
    update_rlist(e);
    e->tpa = e->class_tpa[0];
    for (int c = NC - 1; c >= 0; --c)
        if (e->class_ntiles[c]) { e->tpa = e->class_tpa[c]; break; }
    d.tpa = e->tpa;

    CU(cudaMemcpyAsync(d.tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, e->stream));
    d.nchunks = (int)chunks.size();
    CU(cudaMemcpyAsync(d.chunks, chunks.data(), chunks.size() * sizeof(int4), cudaMemcpyHostToDevice, e->stream));
    CU(cudaMemcpyAsync(d.tile_order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    CU(cudaMemcpyAsync(d.cell_rep, cell_rep.data(), cell_rep.size() * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    CU(cudaMemsetAsync(d.cell_count, 0, ncells * sizeof(int), e->stream));
    CU(cudaMemsetAsync(d.max_needed, 0, sizeof(int), e->stream));
    CU(cudaMemsetAsync(e->trace_buf, 0, TR_SLOTS * sizeof(unsigned long long), e->stream));
    d.trace = (e->cfg.flags & MDGB_FLAG_TRACE) ? e->trace_buf : nullptr;
    CU(cudaMemsetAsync(d.err, 0, 2 * sizeof(int), e->stream));
    CU(cudaMemsetAsync(d.bar, 0, 8 * sizeof(unsigned int), e->stream));
    CU(cudaMemsetAsync(d.rb, 0, (4 + 3 * (size_t)nrep) * sizeof(int), e->stream));
    CU(cudaMemcpyAsync(d.rep, e->rep_host.data(), nrep * sizeof(RepDev), cudaMemcpyHostToDevice, e->stream));
    // the caller's arrays: read by the scatter kernel where they lie (the
    // GPU reaches pageable host memory), else copied to the device staging
    // first.  Either way they are done with before this call returns (the
    // list rebuild below synchronises).
    const double* dpos = pos;
    const double* vptr = vel;
    const uint16_t* tptr = type;
    const int* rptr = ntypes > 1 ? rank.data() : nullptr;
    if (!e->host_direct) {
        double* spos = e->d_out;
        double* svel = e->d_out + 3 * (size_t)N;
        CU(cudaMemcpyAsync(spos, pos, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice, e->stream));
        if (vel) CU(cudaMemcpyAsync(svel, vel, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice, e->stream));
        CU(cudaMemcpyAsync(e->d_in_t, type, (size_t)N * sizeof(uint16_t), cudaMemcpyHostToDevice, e->stream));
        if (ntypes > 1)
            CU(cudaMemcpyAsync(e->d_in_i, rank.data(), (size_t)N * sizeof(int), cudaMemcpyHostToDevice, e->stream));
        dpos = spos;
        vptr = vel ? svel : nullptr;
        tptr = e->d_in_t;
        rptr = ntypes > 1 ? e->d_in_i : nullptr;
    }
    int nt = ntypes;
    void* args[] = {(void*)&e->dev, (void*)&dpos, (void*)&vptr, (void*)&tptr, (void*)&rptr, (void*)&nt};
    CU(cudaLaunchKernel((const void*)k_scatter_in, dim3((N + 255) / 256), dim3(256), args, 0, e->stream));
    // the kernel may read the caller's arrays and the local rank table: done
    // before anything below can return
    if (e->host_direct && ntypes > 1) CU(cudaStreamSynchronize(e->stream));
    e->thermo_on = e->baro_on = e->thermo_nh = false;
    if (ntypes == 1) {   // the type ids were checked on the device
        int flags = 0;
        rc = read_err(e, &flags);
        if (rc) return rc;
        if (flags) return check_flags(e, flags);
    }
    e->has_state = true;
    // bin and build lists now, so a bare mdgb_step starts from a valid list
    return rebuild_lists(e);
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

// The requested arrays gathered into the caller's order on the device, then
// copied straight into the caller's buffers (pageable memory is fine).
int download_impl(mdgb_engine* e, double* pos, double* vel, double* force, double* pot, double* temp,
                  double* boxes) {
    if (!e->has_state) return fail(e, MDGB_ERR_NO_STATE, "no state uploaded");
    const size_t N = e->ntot;
    double* o = e->d_out;
    double* op = pos ? o : nullptr;
    double* ov = vel ? o + 3 * N : nullptr;
    double* of = force ? o + 6 * N : nullptr;
    double* oe = pot ? o + 9 * N : nullptr;
    double* ot = temp ? o + 10 * N : nullptr;
    if (op || ov || of || oe || ot) {
        void* args[] = {(void*)&e->dev, (void*)&op, (void*)&ov, (void*)&of, (void*)&oe, (void*)&ot};
        CU(cudaLaunchKernel((const void*)k_gather_out, dim3((unsigned)((N + 255) / 256)), dim3(256), args, 0,
                            e->stream));
    }
    if (pos) CU(cudaMemcpyAsync(pos, op, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    if (vel) CU(cudaMemcpyAsync(vel, ov, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    if (force) CU(cudaMemcpyAsync(force, of, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    if (pot) CU(cudaMemcpyAsync(pot, oe, N * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    if (temp) CU(cudaMemcpyAsync(temp, ot, N * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    if (boxes)
        CU(cudaMemcpyAsync(e->rep_host.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost,
                           e->stream));
    CU(cudaStreamSynchronize(e->stream));
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
    for (int c = 0; c < 3; ++c) {
        if (aux[c]) cudaStreamDestroy(aux[c]);
        if (join_ev[c]) cudaEventDestroy(join_ev[c]);
    }
    if (fork_ev) cudaEventDestroy(fork_ev);
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
    {
        int pageable = 0, host_tables = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c.device);
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, c.device);
        e->host_direct = pageable == 1 && host_tables == 1;
    }
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) { delete e; return MDGB_ERR_CUDA; }
    for (int c = 0; c < mdgb_engine::NCLASS; ++c)
        if (cudaStreamCreateWithFlags(&e->aux[c], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&e->join_ev[c], cudaEventDisableTiming) != cudaSuccess) {
            delete e;
            return MDGB_ERR_CUDA;
        }
    if (cudaEventCreateWithFlags(&e->fork_ev, cudaEventDisableTiming) != cudaSuccess) { delete e; return MDGB_ERR_CUDA; }
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
        e->lists_fresh = false;
        // a changed cutoff needs lists built with the new radius
        CU(cudaMemcpyAsync(e->rep_host.data(), e->dev.rep, e->nrep * sizeof(RepDev), cudaMemcpyDeviceToHost,
                           e->stream));
        CU(cudaStreamSynchronize(e->stream));
        for (int r = 0; r < e->nrep; ++r) {
            e->rep_host[r].rebuild = 1;
            e->rep_host[r].rlist = e->rcmax + class_skin_of(e, e->class_of[r]);
        }
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
    if (force) CU(cudaMemcpyAsync(d_f, force, 3 * N * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    if (potential) CU(cudaMemcpyAsync(d_p, potential, N * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    if (temp) CU(cudaMemcpyAsync(d_t, temp, N * sizeof(double), cudaMemcpyHostToDevice, e->stream));
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

MDGB_API int mdgb_prepare_step(mdgb_engine* e, int64_t nsteps, double dt, const mdgb_thermostat* thermostat,
                               const mdgb_barostat* barostat) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    if (e->nrep != 1 && e->has_state) return fail(e, MDGB_ERR_INVALID_ARGUMENT, "ensemble engine: use mdgb_ensemble_prepare");
    cudaSetDevice(e->device);
    const bool nh = thermostat && thermostat->kind == MDGB_THERMOSTAT_NOSE_HOOVER;
    return prepare_impl(e, nsteps, dt, thermostat != nullptr, barostat != nullptr, nh);
}

MDGB_API int mdgb_ensemble_prepare(mdgb_engine* e, int64_t nsteps, double dt) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return prepare_impl(e, nsteps, dt, e->thermo_on, e->baro_on, e->thermo_nh);
}

MDGB_API int mdgb_test_barrier_timeout(mdgb_engine* e, int hold_block, int64_t wait_cycles) {
    if (!e || hold_block < 0 || wait_cycles <= 0) return MDGB_ERR_INVALID_ARGUMENT;
    e->test_hold_block = hold_block;
    e->test_barrier_cycles = wait_cycles;
    return MDGB_OK;
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
        unsigned int direct = 0;
        if (cudaMemcpy(&direct, e->dev.bar + 5, sizeof(direct), cudaMemcpyDeviceToHost) == cudaSuccess)
            e->st.direct_list_builds = direct;
    }
    e->st.neighbor_capacity = e->cap;
    e->st.threads_per_atom = e->tpa;
    for (int c = 0; c < mdgb_engine::NCLASS; ++c) {
        e->st.class_threads_per_atom[c] = e->class_tpa[c];
        e->st.class_replicas[c] = e->class_nrep[c];
        e->st.class_skin[c] = class_skin_of(e, c);
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
        cudaMemset(e->dev.bar + 5, 0, sizeof(unsigned int));
    }
    return MDGB_OK;
}

MDGB_API int mdgb_synchronize(mdgb_engine* e) {
    if (!e) return MDGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return cudaStreamSynchronize(e->stream) == cudaSuccess ? MDGB_OK : MDGB_ERR_CUDA;
}

}  // extern "C"
