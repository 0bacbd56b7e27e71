// kernels_step.cu -- the per-step O(N) work of the engine in one cooperative
// persistent kernel (k_pre), plus the macro-parameter reduction kernel.
//
//   [coupling]  reductions -> Berendsen lambda / mu
//               (solver/src/initializer/thermostat.rs:24-34, barostat.rs:21-31,
//                solver/src/macro_parameters/{mod,energy,pressure,temperature}.rs):
//               exact 128-bit fixed-point sums on the mixed path (integer
//               work, phase_partials_fx), FP64 trees (or the reference's
//               serial order) on the FP64 path
//   [drift]     v += F dt/2m, thermostat scale, pending barostat scale of x,
//               x += v dt, periodic wrap, FP32 mirror, displacement
//               (solver/src/solver/integrator.rs:30-47, core/src/particle.rs:120-141)
//   [rebuild]   per replica, only when the displacement (or a forced rebuild)
//               asks for it: integer counting sort of atoms into cells
//               (count -> exclusive scan -> scatter -> canonical order inside
//               each cell); the Verlet list of brute-mode replicas here, of
//               cell-mode replicas in k_build_list (kernels_list.cu), which
//               follows every k_pre launch.
//   After a force pass that already kicked and drifted (NVE chunks), k_pre
//   only takes the rebuild decision -- without a grid barrier when no replica
//   needs one -- and rebuilds if needed.
//
// On the mixed path the FP64 integration uses fused multiply-adds (explicit
// __fma_rn); the FP64 path keeps the reference's separate multiply and add.
//
// Phases are separated by a bounded grid barrier (the kernel is launched
// cooperatively, so every block is resident).  A barrier that waits longer
// than ~2 s sets E_TIMEOUT and the launch ends: every block stops at its next
// barrier at the latest, so no phase runs on the incomplete results of the
// one before (and the engine puts the chunk's starting state back).  Every
// index derived from scratch data is range-checked as well.  Data produced by
// another block inside the same launch is read with ld.global.cg (L2), never
// from a possibly stale L1 line.
//
// This file is compiled with -fmad=false: its FP64 arithmetic (kick, drift,
// wrap, reductions, coupling factors) keeps the reference's unfused
// multiply-then-add rounding unless a fused operation is written out.
#include "mdgb_internal.cuh"

namespace mdgb {

constexpr long long BARRIER_LIMIT_CYCLES = 4000000000LL;
constexpr double K_B = 1.380648528;  // core/src/lib.rs:15

static_assert(sizeof(RepDev) % 8 == 0, "RepDev must be a whole number of 8-byte words");


// One replica record per block, in shared memory (phases work tile by tile
// and a tile never straddles replicas).  The copy is kept while consecutive
// tiles of a block belong to the same replica and dropped at every grid
// barrier (the next phase may see fields the previous one changed).
__shared__ RepDev g_tile_rep;
__shared__ int g_tile_rep_id;

__device__ __forceinline__ void tile_rep_reset() {
    if (threadIdx.x == 0) g_tile_rep_id = -1;
    __syncthreads();
}

__device__ __forceinline__ const RepDev& tile_rep(const Dev& d, int r) {
    if (g_tile_rep_id == r) return g_tile_rep;   // block-uniform
    __syncthreads();  // every thread is done with the previous tile's record
    const long long* src = reinterpret_cast<const long long*>(d.rep + r);
    long long* dst = reinterpret_cast<long long*>(&g_tile_rep);
    for (int i = threadIdx.x; i < (int)(sizeof(RepDev) / 8); i += blockDim.x) dst[i] = __ldcg(src + i);
    if (threadIdx.x == 0) g_tile_rep_id = r;
    __syncthreads();
    return g_tile_rep;
}

__device__ __forceinline__ double4_32a ldcg4(const double4_32a* p) {
    const double2 a = __ldcg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldcg(reinterpret_cast<const double2*>(p) + 1);
    return make_double4_32a(a.x, a.y, b.x, b.y);
}

// The grid barrier's wait limit in clock cycles (set at kernel entry) and the
// block's verdict after the last barrier.
__shared__ long long g_bar_limit;
__shared__ int g_bar_abort;

__device__ __forceinline__ void barrier_setup(const StepParams& sp) {
    if (threadIdx.x == 0) {
        g_bar_limit = sp.barrier_cycles > 0 ? sp.barrier_cycles : BARRIER_LIMIT_CYCLES;
        g_bar_abort = 0;
    }
}

// Returns true when the launch must stop: this block's wait ran out, or
// another block's did (E_TIMEOUT in the error word).  A block that stops
// does no work of the next phase, so no phase ever reads the incomplete
// results of the one before; every block ends at its next barrier at the
// latest, each wait being bounded.  Call sites: if (grid_barrier(d)) return;
__device__ __forceinline__ bool grid_barrier(const Dev& d) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* gen = d.bar + 1;
        const unsigned int g = *gen;
        __threadfence();
        const unsigned int arrived = atomicAdd(d.bar, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(d.bar, 0u);
            __threadfence();
            atomicAdd(d.bar + 1, 1u);
        } else {
            const long long t0 = clock64();
            while (*gen == g) {
                __nanosleep(100);
                if (clock64() - t0 > g_bar_limit) {
                    atomicOr(d.err, E_TIMEOUT);
                    break;
                }
            }
        }
        __threadfence();
        g_tile_rep_id = -1;
        g_bar_abort = (*(volatile int*)d.err & E_TIMEOUT) ? 1 : 0;
    }
    __syncthreads();
    return g_bar_abort != 0;
}

// Deterministic block sum of NV doubles (fixed shuffle tree, fixed warp order).
// Result valid in thread 0.
// Warp stage: a reduce-scatter butterfly -- at offsets 16, 8, ... each lane
// keeps half of its values and adds the partner's copy of that half, so after
// log2(NV) stages lane L holds one value index (bits of L) and the remaining
// offsets finish plain sums: NV - 1 + log2(32/NV) FP64 adds per lane instead
// of 5 NV (the FP64 pipe is narrow on GB300).  NV is a power of two <= 32.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sm) {
    static_assert(NV >= 1 && NV <= 32 && (NV & (NV - 1)) == 0, "power of two");
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int idx = 0;
#pragma unroll
    for (int c = NV, o = 16; c > 1; c >>= 1, o >>= 1) {
        const bool hb = (lane & o) != 0;
#pragma unroll
        for (int k = 0; k < c / 2; ++k) {
            const double send = hb ? v[k] : v[c / 2 + k];
            const double keep = hb ? v[c / 2 + k] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
        if (hb) idx += c / 2;
    }
#pragma unroll
    for (int o = 16 / NV; o > 0; o >>= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
    __syncthreads();
    if ((lane & (32 / NV - 1)) == 0) sm[idx * 32 + w] = v[0];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = sm[k * 32];
            for (int i = 1; i < nw; ++i) s += sm[k * 32 + i];
            v[k] = s;
        }
    }
    __syncthreads();
}

__device__ __forceinline__ float block_max(float v, float* sm) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, off));
    __syncthreads();
    if (lane == 0) sm[w] = v;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int i = 1; i < nw; ++i) v = fmaxf(v, sm[i]);
    __syncthreads();
    return v;
}

__device__ __forceinline__ int block_max_int(int v, int* sm) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, off));
    __syncthreads();
    if (lane == 0) sm[w] = v;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int i = 1; i < nw; ++i) v = max(v, sm[i]);
    __syncthreads();
    return v;
}

// Two-level deterministic reduction of tile partials: one warp per chunk of
// <= CHUNK_TILES tiles (phase_chunk_sums), then one warp per replica over its
// chunks -- a replica of millions of atoms is summed by many warps in
// parallel, always in the same order.
// Rows of 8 partials (one per tile or chunk, 64 bytes) summed slot by slot by
// one warp: lane l adds rows l, l + 32, ... in order, then a shuffle tree per
// slot.  Each lane loads a row's slots together (four 16-byte loads), so the
// loads of all slots are in flight at once.  Result valid in lane 0.
template <int NS>
__device__ __forceinline__ void warp_sum_rows(const double* rows, int n, double (&s)[NS]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < NS; ++k) s[k] = 0.0;
    for (int t = lane; t < n; t += 32) {
        const double2* row = reinterpret_cast<const double2*>(rows + (size_t)t * 8);
        double v[8];
#pragma unroll
        for (int q = 0; q < (NS + 1) / 2; ++q) {
            const double2 x = __ldcg(row + q);
            v[2 * q] = x.x; v[2 * q + 1] = x.y;
        }
#pragma unroll
        for (int k = 0; k < NS; ++k) s[k] += v[k];
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s[k] += __shfl_down_sync(0xffffffffu, s[k], off);
    }
}

template <int NS>
__device__ void phase_chunk_sums(const Dev& d) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int c = gw; c < d.nchunks; c += nw) {
        const int4 ch = d.chunks[c];
        double s[NS];
        warp_sum_rows<NS>(d.part + (size_t)ch.y * 8, ch.z, s);
        if (lane == 0)
            for (int k = 0; k < NS; ++k) d.cpart[(size_t)c * 8 + k] = s[k];
    }
}

// Sums over the chunk partials of one replica by one warp (fixed order),
// slots 0..NS-1, broadcast to every lane.
template <int NS>
__device__ __forceinline__ void warp_sum_tiles(const Dev& d, const RepDev& R, double (&S)[NS]) {
    warp_sum_rows<NS>(d.cpart + (size_t)R.chunk_begin * 8, R.nchunks, S);
#pragma unroll
    for (int k = 0; k < NS; ++k) S[k] = __shfl_sync(0xffffffffu, S[k], 0);
}


// ---------------------------------------------------------------------------
// Tree-order reductions over atoms of type `sel` (all of one mass m, so m is
// factored out of the sums and applied once per replica; halving is exact
// and applied once too -- fewer FP64-pipe operations per atom).
// Pass 1 slots: 0-2 sum(v), 3 count, 4 sum(temp), 5 sum(v.v), 6 sum(potential).
// One atom's inputs of pass 1, loaded a tile ahead (a block walks its tiles
// one after another; the loads of the next overlap this one's sums).
struct Pass1In {
    int ty;
    double vx, vy, vz, vir, pot;
};

__device__ __forceinline__ void pass1_load(const Dev& d, int s, Pass1In& in) {
    const int N = d.ntot;
    in.ty = (int)__ldcg(reinterpret_cast<const long long*>(d.pos + s) + 3);
    in.vx = __ldcg(d.vel + s); in.vy = __ldcg(d.vel + N + s); in.vz = __ldcg(d.vel + 2 * N + s);
    in.vir = __ldcg(d.evir + s);
    in.pot = __ldcg(d.epot + s);
}

__device__ void phase_partials1(const Dev& d, int sel) {
    __shared__ double sm[8 * 32];
    int t = blockIdx.x;
    int4 tl = t < d.ntiles ? d.tiles[t] : make_int4(0, 0, 0, 0);
    Pass1In cur;
    cur.ty = -1;
    if (t < d.ntiles && (int)threadIdx.x < tl.z) pass1_load(d, tl.y + threadIdx.x, cur);
    for (; t < d.ntiles; t += gridDim.x) {
        const int tn = t + gridDim.x;
        int4 tln = make_int4(0, 0, 0, 0);
        Pass1In nxt;
        nxt.ty = -1;
        if (tn < d.ntiles) {
            tln = d.tiles[tn];
            if ((int)threadIdx.x < tln.z) pass1_load(d, tln.y + threadIdx.x, nxt);
        }
        double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if ((int)threadIdx.x < tl.z && cur.ty == sel) {
            const double vx = cur.vx, vy = cur.vy, vz = cur.vz;
            v[0] = vx; v[1] = vy; v[2] = vz; v[3] = 1.0;
            v[4] = cur.vir;
            v[5] = vx * vx + vy * vy + vz * vz;
            v[6] = cur.pot;
        }
        block_sum<8>(v, sm);
        if (threadIdx.x == 0)
            for (int k = 0; k < 8; ++k) d.part[(size_t)t * 8 + k] = v[k];
        tl = tln;
        cur = nxt;
    }
}

// One warp per replica: COM velocity, momentum, kinetic and potential energy
// (mod.rs:12-34, energy.rs:14-49).
__device__ void phase_finalize1(const Dev& d, int sel) {
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const double m = d.mass[sel];
    for (int r = gw; r < d.nrep; r += warps) {
        const RepDev R = load_rep(d.rep + r);
        double S[7];
        warp_sum_tiles<7>(d, R, S);
        if ((threadIdx.x & 31) == 0) {
            RepDev* W = d.rep + r;
            W->vcm[0] = S[0] / S[3]; W->vcm[1] = S[1] / S[3]; W->vcm[2] = S[2] / S[3];
            W->mom[0] = S[0] * m; W->mom[1] = S[1] * m; W->mom[2] = S[2] * m;
            W->msum = S[3] * m; W->virsum = S[4]; W->ke = 0.5 * (m * S[5]); W->pe = S[6] * 0.5;
            W->count = (long long)S[3];
        }
    }
}

// Pass 2 slot 0: sum(|v - vcm|^2)
__device__ void phase_partials2(const Dev& d, int sel) {
    __shared__ double sm[1 * 32];
    const int N = d.ntot;
    for (int t = blockIdx.x; t < d.ntiles; t += gridDim.x) {
        const int4 tl = d.tiles[t];
        const int s = tl.y + threadIdx.x;
        double v[1] = {0};
        if ((int)threadIdx.x < tl.z) {
            const int ty = (int)__ldcg(reinterpret_cast<const long long*>(d.pos + s) + 3);
            if (ty == sel) {
                const double vc0 = __ldcg(&d.rep[tl.x].vcm[0]), vc1 = __ldcg(&d.rep[tl.x].vcm[1]),
                             vc2 = __ldcg(&d.rep[tl.x].vcm[2]);
                const double dx = __ldcg(d.vel + s) - vc0, dy = __ldcg(d.vel + N + s) - vc1,
                             dz = __ldcg(d.vel + 2 * N + s) - vc2;
                v[0] = dx * dx + dy * dy + dz * dz;
            }
        }
        block_sum<1>(v, sm);
        if (threadIdx.x == 0) d.part[(size_t)t * 8] = v[0];
    }
}

// temperature.rs:4-7
__device__ __forceinline__ double temperature_of(double thermal, long long n) {
    const double t = (2.0 * thermal) / (3.0 * (double)n * K_B);
    return t * 100.0;
}

// Coupling factors from the reduced T and P (thermostat.rs:31-39, barostat.rs:29-30).
__device__ __forceinline__ void coupling_factors(RepDev* W, const RepDev& R, double T, double P,
                                                 double dt) {
    if (R.thermo_on) {
        if (R.thermo_kind == 0) {
            const double l2 = 1.0 + dt / R.th_tau * (R.th_T0 / T - 1.0);
            W->lambda = sqrt(l2);
        } else {
            const double psi_dot = -((R.th_T0 / T) - 1.0) / R.th_tau;
            const double psi = R.psi + psi_dot * (dt / 2.0);
            W->psi = psi;
            W->lambda = exp(-psi * dt / 2.0);
        }
    }
    if (R.baro_on) {
        const double m3 = 1.0 + dt * R.ba_beta / R.ba_tau * (P - R.ba_P0);
        W->myu = cbrt(m3);
    }
}

// Finalize pass 2.  coupling: first apply the box part of the pending
// barostat update (box *= mu once per type, barostat.rs:45), then T, P and
// the coupling factors.
__device__ void phase_finalize2(const Dev& d, const StepParams& sp, bool coupling, int sel) {
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (int r = gw; r < d.nrep; r += warps) {
        const RepDev R = load_rep(d.rep + r);
        double S1[1];
        warp_sum_tiles<1>(d, R, S1);
        const double sdv = S1[0];
        const double p1 = d.mass[sel] * sdv;              // sum m |v - vcm|^2 (pressure.rs:13-17)
        const double th = 0.5 * p1;                        // energy.rs:25-37
        if ((threadIdx.x & 31) == 0) {
            RepDev* W = d.rep + r;
            double box[3] = {R.box[0], R.box[1], R.box[2]};
            if (coupling && R.pending != 1.0) {
                for (int k = 0; k < d.ntypes; ++k)
                    for (int a = 0; a < 3; ++a) box[a] *= R.pending;
                for (int a = 0; a < 3; ++a) { W->box[a] = box[a]; W->cs[a] = box[a] / (double)R.nc[a]; }
            }
            const double volume = box[0] * box[1] * box[2];
            const double T = temperature_of(th, R.count);
            const double P = (p1 + (-R.virsum) * 0.5) / volume / 3.0;
            W->thermal = th; W->T = T; W->P = P;
            if (coupling) coupling_factors(W, R, T, P, sp.dt);
        }
    }
}

// Mixed path, coupled steps: one pass.  sum_i |v_i - vcm|^2 = sum |v_i|^2 -
// n |vcm|^2 (as sum v_i = n vcm), so pass 2 and its barriers fold into the
// finalize of pass 1; then what phase_finalize2 does (box, T, P, coupling).
// The FP64 path keeps the reference's explicit second pass.
__device__ void phase_finalize_single(const Dev& d, const StepParams& sp, int sel) {
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const double m = d.mass[sel];
    for (int r = gw; r < d.nrep; r += warps) {
        const RepDev R = load_rep(d.rep + r);
        double S[7];
        warp_sum_tiles<7>(d, R, S);
        if ((threadIdx.x & 31) == 0) {
            RepDev* W = d.rep + r;
            const double vc[3] = {S[0] / S[3], S[1] / S[3], S[2] / S[3]};
            W->vcm[0] = vc[0]; W->vcm[1] = vc[1]; W->vcm[2] = vc[2];
            W->mom[0] = S[0] * m; W->mom[1] = S[1] * m; W->mom[2] = S[2] * m;
            W->msum = S[3] * m; W->virsum = S[4]; W->ke = 0.5 * (m * S[5]); W->pe = S[6] * 0.5;
            W->count = (long long)S[3];
            const double p1 = m * (S[5] - S[3] * (vc[0] * vc[0] + vc[1] * vc[1] + vc[2] * vc[2]));
            const double th = 0.5 * p1;
            double box[3] = {R.box[0], R.box[1], R.box[2]};
            if (R.pending != 1.0) {
                for (int k = 0; k < d.ntypes; ++k)
                    for (int a = 0; a < 3; ++a) box[a] *= R.pending;
                for (int a = 0; a < 3; ++a) { W->box[a] = box[a]; W->cs[a] = box[a] / (double)R.nc[a]; }
            }
            const double volume = box[0] * box[1] * box[2];
            const double T = temperature_of(th, (long long)S[3]);
            const double P = (p1 + (-S[4]) * 0.5) / volume / 3.0;
            W->thermal = th; W->T = T; W->P = P;
            coupling_factors(W, R, T, P, sp.dt);
        }
    }
}

// ---------------------------------------------------------------------------
// Exact sums for the mixed path's coupled steps (replaces the FP64 tree of
// passes partials1 / chunk sums there).  A double x = m 2^(e - 1075)
// (m < 2^53) goes onto the binary grid of its tile, unit 2^(T - 1075 - FX_K)
// with T the largest exponent of that quantity in the tile, as a 128-bit
// integer; tiles, then chunks, then replicas are added exactly after
// aligning to the larger grid (bits below 2^-96 of the largest value drop,
// toward zero).  Integer work only -- GB300's FP64 pipe is narrow -- and the
// sums do not depend on the order of the additions.  Headroom: a tile sum is
// below 2^104, a chunk sum below 2^112, a replica of up to 2^27 atoms below
// 2^124.
// Below this many atoms the coupled reductions are latency-bound and the
// FP64 tree (fewer dependent steps) is faster; from here on the exact sums
// (no FP64 pipe work) are.
constexpr int FX_MIN_ATOMS = 65536;

__device__ __forceinline__ int fx_exp(double x) {
    const int e = (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7FFull);
    return e ? e : 1;   // subnormals and zero: exponent 1 without the hidden bit
}

__device__ __forceinline__ __int128 fx_place(double x, int T) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FFull);
    unsigned long long m = b & 0x000FFFFFFFFFFFFFull;
    if (e) m |= 1ull << 52;
    const int s = (e ? e : 1) - T + FX_K;
    __int128 v = 0;
    if (s >= 0) v = (__int128)m << s;          // s <= FX_K: below 2^97
    else if (s > -64) v = (__int128)(m >> (-s));
    return (b >> 63) ? -v : v;
}

// v on grid T moved to the coarser grid Tmax >= T, toward zero
__device__ __forceinline__ __int128 fx_align(__int128 v, int T, int Tmax) {
    const int d = Tmax - T;
    if (d == 0) return v;
    if (d >= 127) return 0;
    return v < 0 ? -((-v) >> d) : (v >> d);
}

__device__ __forceinline__ __int128 fx_shfl_xor(__int128 v, int o) {
    const long long lo = __shfl_xor_sync(0xffffffffu, (long long)(unsigned long long)v, o);
    const long long hi = __shfl_xor_sync(0xffffffffu, (long long)(v >> 64), o);
    return (__int128)(((unsigned __int128)(unsigned long long)hi << 64) | (unsigned long long)lo);
}

// x * 2^(T - 1075 - FX_K) rounded to the nearest double (ties to even)
__device__ __forceinline__ double fx_to_double(__int128 v, int T) {
    if (v == 0) return 0.0;
    const bool neg = v < 0;
    const unsigned __int128 u = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
    const unsigned long long hi = (unsigned long long)(u >> 64), lo = (unsigned long long)u;
    const int p = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
    unsigned long long mant;
    int sh = 0;
    if (p <= 52) {
        mant = lo;
    } else {
        sh = p - 52;
        mant = (unsigned long long)(u >> sh);
        const unsigned __int128 rem = u & ((((unsigned __int128)1) << sh) - 1);
        const unsigned __int128 half = ((unsigned __int128)1) << (sh - 1);
        if (rem > half || (rem == half && (mant & 1ull))) ++mant;
        if (mant >> 53) { mant >>= 1; ++sh; }
    }
    const double r = ldexp((double)mant, sh + T - 1075 - FX_K);
    return neg ? -r : r;
}

// Pass 1 of a coupled step on the mixed path: one exact row per tile, one
// warp per tile (four atoms per lane, all their loads issued before any
// arithmetic; no block-wide synchronisation), warps striding over the tiles.
__device__ void phase_partials_fx(const Dev& d, int sel) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int N = d.ntot;
    for (int t = gw; t < d.ntiles; t += nw) {
        const int4 tl = d.tiles[t];
        double vx[4], vy[4], vz[4], vir[4], pot[4];
        bool in[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int a = lane + 32 * k;
            in[k] = a < tl.z;
            const int s = tl.y + (in[k] ? a : 0);
            vx[k] = __ldcg(d.vel + s); vy[k] = __ldcg(d.vel + N + s); vz[k] = __ldcg(d.vel + 2 * N + s);
            vir[k] = __ldcg(d.evir + s); pot[k] = __ldcg(d.epot + s);
            if (!d.single_type && in[k])
                in[k] = (int)__ldcg(reinterpret_cast<const long long*>(d.pos + s) + 3) == sel;
        }
        double v2[4];
        int ex[FX_NQ];
#pragma unroll
        for (int q = 0; q < FX_NQ; ++q) ex[q] = 1;
        int nonfinite = 0;
        unsigned cnt = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (!in[k]) { vx[k] = vy[k] = vz[k] = vir[k] = pot[k] = 0.0; }
            v2[k] = __fma_rn(vz[k], vz[k], __fma_rn(vy[k], vy[k], __dmul_rn(vx[k], vx[k])));
            cnt += __popc(__ballot_sync(0xffffffffu, in[k]));
            const int e[FX_NQ] = {fx_exp(vx[k]), fx_exp(vy[k]), fx_exp(vz[k]), fx_exp(vir[k]), fx_exp(v2[k]),
                                  fx_exp(pot[k])};
#pragma unroll
            for (int q = 0; q < FX_NQ; ++q) {
                nonfinite |= e[q] == 0x7FF;
                ex[q] = max(ex[q], e[q]);
            }
        }
        nonfinite = __reduce_or_sync(0xffffffffu, nonfinite);
        FxRow* row = d.fx_part + t;
#pragma unroll
        for (int q = 0; q < FX_NQ; ++q) {
            const int T = __reduce_max_sync(0xffffffffu, ex[q]);
            __int128 v = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double xk = q == 0 ? vx[k] : q == 1 ? vy[k] : q == 2 ? vz[k] : q == 3 ? vir[k]
                                : q == 4 ? v2[k] : pot[k];
                v += fx_place(xk, T);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += fx_shfl_xor(v, o);
            if (lane == 0) { row->s[q] = v; row->ex[q] = (unsigned short)T; }
        }
        if (lane == 0) { row->count = cnt; row->nonfinite = nonfinite; }
    }
}

// Rows [0, n) added exactly by one warp: lane l takes rows l, l + 32, ...
// (each row read whole, 128 bytes, eight 16-byte loads) onto its own running
// grid, widened when a row needs it; then the lanes' sums onto the warp's
// grid.  The result, valid in every lane, is on the grid of the largest
// exponent.  Deterministic: the same rows always go to the same lanes in the
// same order.
__device__ __forceinline__ FxRow fx_warp_sum(const FxRow* rows, int n, int first = -1, int stride = 32) {
    const int lane = threadIdx.x & 31;
    if (first < 0) first = lane;
    int T[FX_NQ];
    __int128 s[FX_NQ];
#pragma unroll
    for (int q = 0; q < FX_NQ; ++q) { T[q] = 1; s[q] = 0; }
    long long cnt = 0;
    int nf = 0;
    for (int t = first; t < n; t += stride) {
        const longlong2* p = reinterpret_cast<const longlong2*>(rows + t);
        longlong2 w[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) w[k] = __ldcg(p + k);
        // w[0..5]: s[0..5] (low, high 64 bits); w[6]: ex[0..5] and nonfinite; w[7].x: count
        const unsigned long long e03 = (unsigned long long)w[6].x;
        const unsigned long long e45 = (unsigned long long)w[6].y;
        int re[FX_NQ];
        re[0] = (int)(e03 & 0xFFFF); re[1] = (int)((e03 >> 16) & 0xFFFF);
        re[2] = (int)((e03 >> 32) & 0xFFFF); re[3] = (int)(e03 >> 48);
        re[4] = (int)(e45 & 0xFFFF); re[5] = (int)((e45 >> 16) & 0xFFFF);
        nf |= (int)(e45 >> 32);
        cnt += w[7].x;
#pragma unroll
        for (int q = 0; q < FX_NQ; ++q) {
            const longlong2 h = w[q];   // s[q] occupies 16 bytes: lo, hi
            const __int128 v = (__int128)(((unsigned __int128)(unsigned long long)h.y << 64) |
                                          (unsigned long long)h.x);
            if (re[q] > T[q]) { s[q] = fx_align(s[q], T[q], re[q]); T[q] = re[q]; }
            s[q] += fx_align(v, re[q], T[q]);
        }
    }
    FxRow out;
#pragma unroll
    for (int q = 0; q < FX_NQ; ++q) {
        const int Tw = __reduce_max_sync(0xffffffffu, T[q]);
        __int128 v = fx_align(s[q], T[q], Tw);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += fx_shfl_xor(v, o);
        out.s[q] = v;
        out.ex[q] = (unsigned short)Tw;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        nf |= __shfl_xor_sync(0xffffffffu, nf, o);
    }
    out.count = cnt;
    out.nonfinite = nf;
    return out;
}

// The same with a whole block (threads take rows tid, tid + blockDim, ...),
// then the warps' sums combined in a fixed order.  Result valid in thread 0.
__device__ __forceinline__ FxRow fx_block_sum(const FxRow* rows, int n) {
    __shared__ FxRow sm_w[TILE / 32];   // k_pre and k_macro blocks have TILE threads
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    FxRow r = fx_warp_sum(rows, n, (int)threadIdx.x, (int)blockDim.x);
    __syncthreads();   // a previous call's rows are read
    if (lane == 0) sm_w[w] = r;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < nw; ++i) {
            const FxRow& o = sm_w[i];
#pragma unroll
            for (int q = 0; q < FX_NQ; ++q) {
                const int T = max((int)r.ex[q], (int)o.ex[q]);
                r.s[q] = fx_align(r.s[q], r.ex[q], T) + fx_align(o.s[q], o.ex[q], T);
                r.ex[q] = (unsigned short)T;
            }
            r.count += o.count;
            r.nonfinite |= o.nonfinite;
        }
    }
    return r;
}

// One block per chunk of tile rows.
__device__ void phase_chunk_sums_fx(const Dev& d) {
    for (int c = blockIdx.x; c < d.nchunks; c += gridDim.x) {
        const int4 ch = d.chunks[c];
        const FxRow r = fx_block_sum(d.fx_part + ch.y, ch.z);
        if (threadIdx.x == 0) d.fx_cpart[c] = r;
    }
}

// Mixed path, coupled steps: the replica's exact sums as doubles, then what
// phase_finalize2 does (box, T, P, coupling).  sum_i |v_i - vcm|^2 = sum
// |v_i|^2 - n |vcm|^2 (as sum v_i = n vcm): one pass over the atoms.
__device__ void phase_finalize_fx(const Dev& d, const StepParams& sp, int sel) {
    const double m = d.mass[sel];
    for (int r = blockIdx.x; r < d.nrep; r += gridDim.x) {   // one block per replica
        const RepDev R = load_rep(d.rep + r);
        const FxRow F = fx_block_sum(d.fx_cpart + R.chunk_begin, R.nchunks);
        if (threadIdx.x == 0) {
            double S[7];
            const double nan = __longlong_as_double(0x7FF8000000000000ll);
            S[0] = fx_to_double(F.s[0], F.ex[0]); S[1] = fx_to_double(F.s[1], F.ex[1]);
            S[2] = fx_to_double(F.s[2], F.ex[2]); S[3] = (double)F.count;
            S[4] = fx_to_double(F.s[3], F.ex[3]); S[5] = fx_to_double(F.s[4], F.ex[4]);
            S[6] = fx_to_double(F.s[5], F.ex[5]);
            if (F.nonfinite)
                for (int k = 0; k < 7; ++k) if (k != 3) S[k] = nan;
            RepDev* W = d.rep + r;
            const double vc[3] = {S[0] / S[3], S[1] / S[3], S[2] / S[3]};
            W->vcm[0] = vc[0]; W->vcm[1] = vc[1]; W->vcm[2] = vc[2];
            W->mom[0] = S[0] * m; W->mom[1] = S[1] * m; W->mom[2] = S[2] * m;
            W->msum = S[3] * m; W->virsum = S[4]; W->ke = 0.5 * (m * S[5]); W->pe = S[6] * 0.5;
            W->count = F.count;
            const double p1 = m * (S[5] - S[3] * (vc[0] * vc[0] + vc[1] * vc[1] + vc[2] * vc[2]));
            const double th = 0.5 * p1;
            double box[3] = {R.box[0], R.box[1], R.box[2]};
            if (R.pending != 1.0) {
                for (int k = 0; k < d.ntypes; ++k)
                    for (int a = 0; a < 3; ++a) box[a] *= R.pending;
                for (int a = 0; a < 3; ++a) { W->box[a] = box[a]; W->cs[a] = box[a] / (double)R.nc[a]; }
            }
            const double volume = box[0] * box[1] * box[2];
            const double T = temperature_of(th, F.count);
            const double P = (p1 + (-S[4]) * 0.5) / volume / 3.0;
            W->thermal = th; W->T = T; W->P = P;
            coupling_factors(W, R, T, P, sp.dt);
        }
    }
}

// thermostat.rs:59-65: psi += psi_dot(T') * dt/2 with T' the temperature
// after the first kick, before the velocity scaling.
__device__ __forceinline__ void nh_update_psi(RepDev* W, const RepDev& R, double T, double dt) {
    if (!R.thermo_on || R.thermo_kind != 1) return;
    const double psi_dot = -((R.th_T0 / T) - 1.0) / R.th_tau;
    W->psi = R.psi + psi_dot * (dt / 2.0);
}

__device__ void phase_finalize_nh(const Dev& d, const StepParams& sp, int sel) {
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (int r = gw; r < d.nrep; r += warps) {
        const RepDev R = load_rep(d.rep + r);
        double S1[1];
        warp_sum_tiles<1>(d, R, S1);
        const double sdv = S1[0];
        if ((threadIdx.x & 31) == 0) nh_update_psi(d.rep + r, R, temperature_of(0.5 * (d.mass[sel] * sdv), R.count), sp.dt);
    }
}

// Reference-order reductions: one thread per replica walks the atoms of type
// `sel` in the reference's order and sums serially, exactly as the iterator
// folds of macro_parameters/*.rs do.
__device__ void phase_serial(const Dev& d, const StepParams& sp, int sel, bool coupling, bool nh_after_kick = false) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = gridDim.x * blockDim.x;
    const int N = d.ntot;
    for (int r = gt; r < d.nrep; r += nt) {
        const RepDev R = load_rep(d.rep + r);
        RepDev* W = d.rep + r;
        const long long b = R.begin + R.type_off[sel], e = R.begin + R.type_off[sel + 1];
        const double m = d.mass[sel];
        double sx = 0, sy = 0, sz = 0, sw = 0, ke = 0, pe = 0;
        for (long long k = b; k < e; ++k) {
            const int s = __ldcg(d.slot_of_rank + k);
            if (s < 0 || s >= N) { atomicOr(d.err, E_BOUNDS); continue; }
            const double vx = __ldcg(d.vel + s), vy = __ldcg(d.vel + N + s), vz = __ldcg(d.vel + 2 * N + s);
            sx += vx * m; sy += vy * m; sz += vz * m; sw += 1.0 * m;   // mod.rs:12-25
            ke += m * (vx * vx + vy * vy + vz * vz) / 2.0;              // energy.rs:14-22
            pe += __ldcg(d.epot + s);                                    // energy.rs:40-49
        }
        const double vc[3] = {sx / sw, sy / sw, sz / sw};
        double th = 0, r1 = 0, r2 = 0;
        for (long long k = b; k < e; ++k) {
            const int s = __ldcg(d.slot_of_rank + k);
            if (s < 0 || s >= N) continue;
            const double dx = __ldcg(d.vel + s) - vc[0], dy = __ldcg(d.vel + N + s) - vc[1],
                         dz = __ldcg(d.vel + 2 * N + s) - vc[2];
            th += m * (dx * dx + dy * dy + dz * dz) / 2.0;             // energy.rs:25-37
            r1 += m * dx * dx; r1 += m * dy * dy; r1 += m * dz * dz;   // pressure.rs:13-18
            r2 -= __ldcg(d.evir + s);
        }
        if (nh_after_kick) {
            nh_update_psi(W, R, temperature_of(th, e - b), sp.dt);
            continue;
        }
        double box[3] = {R.box[0], R.box[1], R.box[2]};
        if (coupling && R.pending != 1.0) {
            for (int k = 0; k < d.ntypes; ++k)
                for (int a = 0; a < 3; ++a) box[a] *= R.pending;
            for (int a = 0; a < 3; ++a) { W->box[a] = box[a]; W->cs[a] = box[a] / (double)R.nc[a]; }
        }
        const double volume = box[0] * box[1] * box[2];
        const double T = temperature_of(th, e - b);
        const double P = (r1 + r2 * 0.5) / volume / 3.0;
        W->vcm[0] = vc[0]; W->vcm[1] = vc[1]; W->vcm[2] = vc[2];
        W->mom[0] = sx; W->mom[1] = sy; W->mom[2] = sz;
        W->msum = sw; W->ke = ke; W->pe = pe / 2.0; W->thermal = th; W->virsum = -r2;
        W->count = e - b; W->T = T; W->P = P;
        if (coupling) coupling_factors(W, R, T, P, sp.dt);
    }
}

// psi += psi_dot(T_t) * dt/2 with T_t the temperature of the atoms of type t
// (thermostat.rs:35-39 before the kick, :59-65 after it), per replica with a
// Nose-Hoover thermostat.  Returns true when the launch must stop.
__device__ __forceinline__ bool nh_psi_of_type(const Dev& d, const StepParams& sp, int t) {
    if (d.refmode) {
        phase_serial(d, sp, t, false, true);
        return grid_barrier(d);
    }
    phase_partials1(d, t);
    if (grid_barrier(d)) return true;
    phase_chunk_sums<7>(d);
    if (grid_barrier(d)) return true;
    phase_finalize1(d, t);
    if (grid_barrier(d)) return true;
    phase_partials2(d, t);
    if (grid_barrier(d)) return true;
    phase_chunk_sums<1>(d);
    if (grid_barrier(d)) return true;
    phase_finalize_nh(d, sp, t);
    return grid_barrier(d);
}

// ---------------------------------------------------------------------------
// Drift: integrator.rs:30-47 for every atom; mirror + displacement.
// Nose-Hoover steps: the first kick alone (integrator.rs:30-36), so the
// thermostat can read the temperature between kick and scaling
// (thermostat.rs:47-52,59-65).
// FM (here and in the phases below): the mixed path's fused multiply-adds,
// a compile-time constant -- the callers dispatch on d.mixed once per phase.
template <bool FM>
__device__ void phase_kick(const Dev& d, const StepParams& sp) {
    const int N = d.ntot;
    for (int t = blockIdx.x; t < d.ntiles; t += gridDim.x) {
        const int4 tl = d.tiles[t];
        const int s = tl.y + threadIdx.x;
        if ((int)threadIdx.x >= tl.z) continue;
        const int ty = (int)reinterpret_cast<const long long*>(d.pos + s)[3];
        const double c = sp.kick_c[ty];
        for (int a = 0; a < 3; ++a)
            d.vel[(size_t)a * N + s] = madd(d.vel[(size_t)a * N + s], d.frc[(size_t)a * N + s], c, FM);
    }
}

// Inputs of one atom's drift, loaded one tile ahead (the loop is latency-
// bound: a block walks its tiles one after another).
struct DriftIn {
    double4_32a p;
    double v[3], f[3];
    int cell;
    float4 m0;
};

__device__ __forceinline__ void drift_load(const Dev& d, int s, bool kicked, DriftIn& in) {
    const int N = d.ntot;
    in.p = d.pos[s];
    for (int a = 0; a < 3; ++a) in.v[a] = __ldcg(d.vel + (size_t)a * N + s);
    if (!kicked)
        for (int a = 0; a < 3; ++a) in.f[a] = __ldcg(d.frc + (size_t)a * N + s);
    in.cell = d.cell[s];
    in.m0 = d.mir0[s];
}

template <bool FM>
__device__ void phase_drift(const Dev& d, const StepParams& sp, bool kicked) {
    __shared__ float smx[32];
    __shared__ float tc[7];   // box (FP32), half box, scale since the last rebuild
    const int N = d.ntot;
    constexpr bool fm = FM;
    int tc_rep = -1;          // replica tc[] and disp belong to (block-uniform)
    float disp = 0.f;         // largest displacement seen by this thread in replica tc_rep
    // a contiguous run of tiles per block: the replica (and with it the
    // constants and the displacement maximum) changes only at its boundaries
    const int per = (d.ntiles + gridDim.x - 1) / gridDim.x;
    const int t_end = min(d.ntiles, ((int)blockIdx.x + 1) * per);
    int t = blockIdx.x * per;
    int4 tl = t < t_end ? d.tiles[t] : make_int4(0, 0, 0, 0);
    DriftIn cur;
    if (t < t_end && (int)threadIdx.x < tl.z) drift_load(d, tl.y + threadIdx.x, kicked, cur);
    for (; t < t_end; ++t) {
        // the next tile's inputs in flight while this one computes
        const int tn = t + 1;
        int4 tln = make_int4(0, 0, 0, 0);
        DriftIn nxt;
        if (tn < t_end) {
            tln = d.tiles[tn];
            if ((int)threadIdx.x < tln.z) drift_load(d, tln.y + threadIdx.x, kicked, nxt);
        }
        if (tl.x != tc_rep) {
            if (tc_rep >= 0) {
                const float m = block_max(disp, smx);
                if (threadIdx.x == 0) atomicMax(&d.rep[tc_rep].max_disp_bits, __float_as_uint(m));
                disp = 0.f;
            }
        }
        const RepDev& R = tile_rep(d, tl.x);
        if (tl.x != tc_rep) {
            __syncthreads();
            if (threadIdx.x == 0) drift_consts(R, tc);
            __syncthreads();
            tc_rep = tl.x;
        }
        const int s = tl.y + threadIdx.x;
        if ((int)threadIdx.x < tl.z) {
            double4_32a p = cur.p;
            if (sp.do_drift) {
                const int ty = type_of(p);
                const double c = sp.kick_c[ty];
                double vx = cur.v[0], vy = cur.v[1], vz = cur.v[2];
                if (!kicked) {
                    vx = madd(vx, cur.f[0], c, fm);                      // :30-36 kick
                    vy = madd(vy, cur.f[1], c, fm);
                    vz = madd(vz, cur.f[2], c, fm);
                }
                if (R.thermo_on) {                                       // thermostat.rs:54-58
                    vx = dmul_nospec(vx, R.lambda); vy = dmul_nospec(vy, R.lambda);
                    vz = dmul_nospec(vz, R.lambda);
                }
                d.vel[s] = vx; d.vel[N + s] = vy; d.vel[2 * N + s] = vz;
                double x = p.x, y = p.y, z = p.z;
                if (R.pending != 1.0) {                                  // barostat.rs:46-48
                    x = dmul_nospec(x, R.pending); y = dmul_nospec(y, R.pending);
                    z = dmul_nospec(z, R.pending);
                }
                p.x = x; p.y = y; p.z = z;
                p = drift_wrap(p, vx, vy, vz, sp.dt, R.box, fm);         // :42-46 drift
                d.pos[s] = p;
            }
            const int cl = cur.cell - R.cell_base;
            // cl is out of range only before the first binning (fresh upload);
            // the forced rebuild that follows computes the mirror then.
            if (cl >= 0 && cl < R.nc[0] * R.nc[1] * R.nc[2]) {
                const float4 m = mirror_of(p, cl, R, tc + 3, fm);
                d.mir[s] = m;
                disp = fmaxf(disp, mirror_disp(m, cur.m0, tc));
            }
        }
        tl = tln;
        cur = nxt;
    }
    if (tc_rep >= 0) {
        const float m = block_max(disp, smx);
        if (threadIdx.x == 0) atomicMax(&d.rep[tc_rep].max_disp_bits, __float_as_uint(m));
    }
}

// Per replica: consume the pending barostat factor, decide on a rebuild.
__device__ void phase_decide(const Dev& d, const StepParams& sp) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = gridDim.x * blockDim.x;
    for (int r = gt; r < d.nrep; r += nt) decide_replica(d, sp, r);
}

// ---------------------------------------------------------------------------
// Rebuild phases (only tiles/cells of replicas with rebuild set do work).

// The rebuild work list (block 0; the grid barrier after the zero phase
// publishes it): the rebuilding replicas with prefix offsets of their cells
// (the grid the decide phase set; one cell in brute mode) and tiles, so the
// rebuild phases and the list build visit only their work.  Replicas the
// paired list build does not take come first (pass 0), the others after.
__device__ void phase_work_list(const Dev& d) {
    __shared__ int wsum[3][TILE / 32];
    __shared__ int carry[3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int* rb = d.rb;
    int* ids = rb + 2;
    int* coff = rb + 2 + d.nrep;
    int* toff = rb + 3 + 2 * d.nrep;
    if (threadIdx.x < 3) carry[threadIdx.x] = 0;
    __syncthreads();
    for (int pass = 0; pass < 2; ++pass) {
        for (int base = 0; base < d.nrep; base += blockDim.x) {
            const int r = base + threadIdx.x;
            int v[3] = {0, 0, 0};
            if (r < d.nrep) {
                const RepDev* W = d.rep + r;
                const bool paired = W->n >= LIST_PAIRED_MIN_ATOMS && __ldcg(&W->mode) == MODE_CELLS;
                if (__ldcg(&W->rebuild) && paired == (pass == 1)) {
                    v[0] = 1;
                    v[1] = __ldcg(&W->nc[0]) * __ldcg(&W->nc[1]) * __ldcg(&W->nc[2]);
                    v[2] = W->ntiles;
                }
            }
            int inc[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                inc[q] = v[q];
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, inc[q], off);
                    if (lane >= off) inc[q] += y;
                }
                if (lane == 31) wsum[q][w] = inc[q];
            }
            __syncthreads();
            if (v[0]) {
                int ex[3];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    ex[q] = carry[q] + inc[q] - v[q];
                    for (int k = 0; k < w; ++k) ex[q] += wsum[q][k];
                }
                ids[ex[0]] = r;
                coff[ex[0]] = ex[1];
                toff[ex[0]] = ex[2];
            }
            __syncthreads();
            if (threadIdx.x < 3)
                for (int k = 0; k < (int)(blockDim.x >> 5); ++k) carry[threadIdx.x] += wsum[threadIdx.x][k];
            __syncthreads();
        }
        if (pass == 0 && threadIdx.x == 0) rb[1] = carry[0];
    }
    if (threadIdx.x == 0) {
        rb[0] = carry[0];
        coff[carry[0]] = carry[1];
        toff[carry[0]] = carry[2];
    }
}

__device__ void phase_zero_cells(const Dev& d) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = gridDim.x * blockDim.x;
    for (int c = gt; c < d.ncells; c += nt) {
        const int r = d.cell_rep[c];
        if (__ldcg(&d.rep[r].rebuild)) d.cell_count[c] = 0;
    }
}

// Cell of every atom, and its slot among the cell's atoms in arrival order
// (tmp_i row 3): one counter atomic per distinct cell in a warp -- the atoms
// are mostly still sorted by cell, so a warp covers only a few.
__device__ void phase_bin(const Dev& d) {
    const int N = d.ntot;
    const int lane = threadIdx.x & 31;
    // a contiguous run of the rebuilding replicas' tiles per block (the
    // replica record is fetched only when the run crosses into the next)
    const int m = __ldcg(d.rb), nw = __ldcg(rb_tile_off(d) + m);
    const int per = (nw + gridDim.x - 1) / gridDim.x;
    const int w_end = min(nw, ((int)blockIdx.x + 1) * per);
    int wi = blockIdx.x * per;
    int i = wi < w_end ? rb_locate(rb_tile_off(d), m, wi) - 1 : 0;
    int next = wi, shift = 0;   // where replica i's run ends; tile index - work index inside it
    for (; wi < w_end; ++wi) {
        while (wi >= next) {
            ++i;
            next = __ldcg(rb_tile_off(d) + i + 1);
            shift = d.rep[__ldcg(rb_rep(d) + i)].tile_begin - __ldcg(rb_tile_off(d) + i);
        }
        const int4 tl = d.tiles[wi + shift];
        const RepDev& R = tile_rep(d, tl.x);
        const int s = tl.y + threadIdx.x;
        const bool act = (int)threadIdx.x < tl.z;
        const unsigned am = __ballot_sync(0xffffffffu, act);
        if (!act) continue;
        const double4_32a p = d.pos[s];
        int local = 0;
        if (R.mode == MODE_CELLS) {
            const double x[3] = {p.x, p.y, p.z};
            int c[3];
            for (int a = 0; a < 3; ++a) {
                // wrapped positions are >= 0: truncation is the floor
                const int ci = __double2int_rz(__dmul_rn(x[a], R.inv_cs[a]));
                c[a] = min(max(ci, 0), R.nc[a] - 1);
            }
            local = (c[0] * R.nc[1] + c[1]) * R.nc[2] + c[2];
        }
        const int cell = R.cell_base + local;
        d.tmp_i[2 * (size_t)N + s] = cell;
        const unsigned peers = __match_any_sync(am, cell);
        const int leader = __ffs(peers) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(d.cell_count + cell, __popc(peers));
        base = __shfl_sync(am, base, leader);
        d.tmp_i[3 * (size_t)N + s] = base + __popc(peers & ((1u << lane) - 1u));
    }
}

// Exclusive scan of cell counts over all cells (block chunks + block sums).
__device__ void phase_scan_a(const Dev& d, int chunk) {
    __shared__ double sm[32];
    const int b0 = blockIdx.x * chunk, b1 = min(b0 + chunk, d.ncells);
    double v[1] = {0.0};
    for (int c = b0 + threadIdx.x; c < b1; c += blockDim.x) v[0] += (double)__ldcg(d.cell_count + c);
    block_sum<1>(v, sm);
    if (threadIdx.x == 0) d.bsum[blockIdx.x] = (int)v[0];
}

// Exclusive scan of the per-block sums by block 0 (each thread a contiguous run).
__device__ void phase_scan_b(const Dev& d) {
    __shared__ int part[TILE];
    if (blockIdx.x != 0) return;
    const int G = gridDim.x;
    const int per = (G + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per, b1 = min(b0 + per, G);
    int sum = 0;
    for (int b = b0; b < b1; ++b) sum += __ldcg(d.bsum + b);
    part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int i = 0; i < (int)blockDim.x; ++i) { const int t = part[i]; part[i] = run; run += t; }
        d.cell_start[d.ncells] = run;
    }
    __syncthreads();
    int run = part[threadIdx.x];
    for (int b = b0; b < b1; ++b) {
        const int v = __ldcg(d.bsum + b);
        d.bsum[b] = run;
        run += v;
    }
}

__device__ void phase_scan_c(const Dev& d, int chunk) {
    __shared__ int wsum[32];
    __shared__ int carry;
    const int b0 = blockIdx.x * chunk, b1 = min(b0 + chunk, d.ncells);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = __ldcg(d.bsum + blockIdx.x);
    __syncthreads();
    for (int base = b0; base < b1; base += blockDim.x) {
        const int c = base + threadIdx.x;
        const int x = (c < b1) ? __ldcg(d.cell_count + c) : 0;
        int inc = x;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off) inc += y;
        }
        if (lane == 31) wsum[w] = inc;
        __syncthreads();
        if (threadIdx.x == 0) {
            int run = 0;
            for (int i = 0; i < nw; ++i) { const int t = wsum[i]; wsum[i] = run; run += t; }
        }
        __syncthreads();
        if (c < b1) d.cell_start[c] = carry + wsum[w] + inc - x;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += wsum[w] + inc;
        __syncthreads();
    }
}

// carry_forces: also move frc/epot/evir (a refresh that no force evaluation
// follows); a step's force pass rewrites them after the rebuild anyway.
// One atom's move to the scratch copy: its inputs (ScatterIn, loaded for two
// tiles before either is stored, so a thread has both in flight) and its
// slot, perm[slot] = s.
struct ScatterIn {
    double4_32a p;
    double v[3];
    int cell, slot, orig, rank;
};

__device__ __forceinline__ void scatter_load(const Dev& d, const RepDev& R, int s, ScatterIn& in) {
    const int N = d.ntot;
    in.cell = d.tmp_i[2 * (size_t)N + s];
    const int within = d.tmp_i[3 * (size_t)N + s];
    in.p = d.pos[s];
    for (int k = 0; k < 3; ++k) in.v[k] = d.vel[(size_t)k * N + s];
    in.orig = d.orig[s];
    in.rank = d.rank[s];
    // brute mode: one cell holds the whole replica in its current order
    const bool cell_ok = in.cell >= R.cell_base && in.cell < R.cell_base + R.cell_cap;
    in.slot = R.mode == MODE_BRUTE ? s : (cell_ok ? __ldcg(d.cell_start + in.cell) + within : -1);
    if (!cell_ok) in.cell = -1;
}

__device__ __forceinline__ void scatter_store(const Dev& d, const RepDev& R, int s, const ScatterIn& in,
                                              bool carry_forces) {
    const int N = d.ntot;
    if (in.cell < 0 || in.slot < R.begin || in.slot >= R.begin + R.n) { atomicOr(d.err, E_CELLS); return; }
    d.perm[in.slot] = s;
    d.tmp_pos[s] = in.p;
    for (int k = 0; k < 3; ++k) d.tmp_d[(size_t)k * N + s] = in.v[k];
    if (carry_forces) {
        for (int k = 0; k < 3; ++k) d.tmp_d[(size_t)(3 + k) * N + s] = d.frc[(size_t)k * N + s];
        d.tmp_d[(size_t)6 * N + s] = d.epot[s];
        d.tmp_d[(size_t)7 * N + s] = d.evir[s];
    }
    d.tmp_i[s] = in.orig;
    d.tmp_i[(size_t)N + s] = in.rank;
}

__device__ void phase_scatter(const Dev& d, bool carry_forces) {
    // a contiguous run of the rebuilding replicas' tiles per block (the
    // replica record is fetched only when the run crosses into the next);
    // two tiles of a replica at a time
    const int m = __ldcg(d.rb), nw = __ldcg(rb_tile_off(d) + m);
    const int per = (nw + gridDim.x - 1) / gridDim.x;
    const int w_end = min(nw, ((int)blockIdx.x + 1) * per);
    int wi = blockIdx.x * per;
    int i = wi < w_end ? rb_locate(rb_tile_off(d), m, wi) - 1 : 0;
    int next = wi, shift = 0;   // where replica i's run ends; tile index - work index inside it
    while (wi < w_end) {
        while (wi >= next) {
            ++i;
            next = __ldcg(rb_tile_off(d) + i + 1);
            shift = d.rep[__ldcg(rb_rep(d) + i)].tile_begin - __ldcg(rb_tile_off(d) + i);
        }
        const bool two = wi + 1 < w_end && wi + 1 < next;
        const int4 ta = d.tiles[wi + shift];
        const int4 tb = two ? d.tiles[wi + 1 + shift] : make_int4(0, 0, 0, 0);
        const RepDev& R = tile_rep(d, ta.x);
        const int sa = ta.y + threadIdx.x, sb = tb.y + threadIdx.x;
        const bool aa = (int)threadIdx.x < ta.z, ab = two && (int)threadIdx.x < tb.z;
        ScatterIn xa, xb;
        if (aa) scatter_load(d, R, sa, xa);
        if (ab) scatter_load(d, R, sb, xb);
        if (aa) scatter_store(d, R, sa, xa, carry_forces);
        if (ab) scatter_store(d, R, sb, xb, carry_forces);
        wi += two ? 2 : 1;
    }
}

// Cells of up to 32 * SORT_MAX_PER_LANE atoms are ranked by shuffles; more
// crowded ones by a serial insertion sort.
constexpr int SORT_MAX_PER_LANE = 4;

// The geometry of one replica that the gather needs, read through L2 (the
// decide phase of this launch may have changed the box).
struct CellGeom {
    double box[3], cs[3];
    float hL[3];
    int nc[3];
    int cell_base, mode, n, r;
    long long begin;
};

__device__ __forceinline__ void load_geom(const Dev& d, int r, CellGeom& g) {
    const RepDev* W = d.rep + r;
    for (int a = 0; a < 3; ++a) {
        g.box[a] = __ldcg(&W->box[a]);
        g.cs[a] = __ldcg(&W->cs[a]);
        g.nc[a] = __ldcg(&W->nc[a]);
        g.hL[a] = 0.5f * dbl_to_flt_rn(g.box[a]);
    }
    g.cell_base = __ldcg(&W->cell_base);
    g.mode = __ldcg(&W->mode);
    g.n = __ldcg(&W->n);
    g.begin = __ldcg(&W->begin);
    g.r = r;
}

// Scratch element i (the atom's index before the rebuild) to slot s of cell
// c: its scratch row loaded (gather_load), then written to the slot with a
// fresh mirror (gather_store).
struct GatherIn {
    double4_32a p;
    double v[3];
    int orig, rank;
};

__device__ __forceinline__ void gather_load(const Dev& d, int i, GatherIn& in) {
    const int N = d.ntot;
    in.p = ldcg4(d.tmp_pos + i);
    for (int k = 0; k < 3; ++k) in.v[k] = __ldcg(d.tmp_d + (size_t)k * N + i);
    in.orig = __ldcg(d.tmp_i + i);
    in.rank = __ldcg(d.tmp_i + (size_t)N + i);
}

template <bool FM>
__device__ __forceinline__ void gather_store(const Dev& d, const CellGeom& g, int c, int i, int s,
                                             const GatherIn& in, bool carry_forces) {
    const int N = d.ntot;
    d.pos[s] = in.p;
    for (int k = 0; k < 3; ++k) d.vel[(size_t)k * N + s] = in.v[k];
    if (carry_forces) {
        for (int k = 0; k < 3; ++k) d.frc[(size_t)k * N + s] = __ldcg(d.tmp_d + (size_t)(3 + k) * N + i);
        d.epot[s] = __ldcg(d.tmp_d + (size_t)6 * N + i);
        d.evir[s] = __ldcg(d.tmp_d + (size_t)7 * N + i);
    }
    d.orig[s] = in.orig;
    d.rank[s] = in.rank;
    d.cell[s] = c;
    const float4 m = mirror_of(in.p, c - g.cell_base, g, g.hL, FM);
    d.mir[s] = m;
    d.mir0[s] = m;
    if (in.rank >= 0 && in.rank < N) d.slot_of_rank[in.rank] = s;
    else atomicOr(d.err, E_BOUNDS);
}

__device__ __forceinline__ bool gather_ok(const Dev& d, const CellGeom& g, int i, int s) {
    if (i < g.begin || i >= g.begin + g.n || s < g.begin || s >= g.begin + g.n) {
        atomicOr(d.err, E_BOUNDS);
        return false;
    }
    return true;
}

template <bool FM>
__device__ __forceinline__ void gather_one(const Dev& d, const CellGeom& g, int c, int i, int s,
                                           bool carry_forces) {
    if (!gather_ok(d, g, i, s)) return;
    GatherIn in;
    gather_load(d, i, in);
    gather_store<FM>(d, g, c, i, s, in, carry_forces);
}

// One cell: canonical order (ascending caller index) and the gather.
template <bool FM>
__device__ void sort_gather_cell(const Dev& d, const CellGeom& g, int c, int b, int n, bool carry_forces) {
    const int N = d.ntot;
    const int lane = threadIdx.x & 31;
    if (g.mode == MODE_BRUTE) {
        // the scatter kept the replica's order: slot i holds element i
        for (int k = lane; k < n; k += 32) gather_one<FM>(d, g, c, __ldcg(d.perm + b + k), b + k, carry_forces);
    } else if (n <= 32 * SORT_MAX_PER_LANE) {
        int e[SORT_MAX_PER_LANE], key[SORT_MAX_PER_LANE], rank[SORT_MAX_PER_LANE];
#pragma unroll
        for (int q = 0; q < SORT_MAX_PER_LANE; ++q) {
            const int i = q * 32 + lane;
            e[q] = i < n ? __ldcg(d.perm + b + i) : -1;
            const bool ok = e[q] >= 0 && e[q] < N;
            if (i < n && !ok) atomicOr(d.err, E_BOUNDS);
            key[q] = ok ? __ldcg(d.tmp_i + e[q]) : 0x7FFFFFFF;
            rank[q] = 0;
        }
        if (n <= 32) {
            // one key a lane, n shuffles
            for (int k = 0; k < n; ++k) rank[0] += (__shfl_sync(0xffffffffu, key[0], k) < key[0]) ? 1 : 0;
        } else {
#pragma unroll
            for (int q2 = 0; q2 < SORT_MAX_PER_LANE; ++q2) {
                if (q2 * 32 >= n) break;
                for (int k = 0; k < 32; ++k) {
                    const int kk = __shfl_sync(0xffffffffu, key[q2], k);
#pragma unroll
                    for (int q = 0; q < SORT_MAX_PER_LANE; ++q) rank[q] += (kk < key[q]) ? 1 : 0;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < SORT_MAX_PER_LANE; ++q) {
            const int i = q * 32 + lane;
            if (i < n && e[q] >= 0 && e[q] < N && rank[q] < n) gather_one<FM>(d, g, c, e[q], b + rank[q], carry_forces);
        }
    } else {
        // very crowded cell: serial insertion sort of the slots, then the gather
        if (lane == 0) {
            for (int a = 1; a < n; ++a) {
                const int e0 = __ldcg(d.perm + b + a);
                if (e0 < 0 || e0 >= N) { atomicOr(d.err, E_BOUNDS); break; }
                const int k0 = __ldcg(d.tmp_i + e0);
                int k = a - 1;
                while (k >= 0) {
                    const int f = __ldcg(d.perm + b + k);
                    if (f < 0 || f >= N || __ldcg(d.tmp_i + f) <= k0) break;
                    d.perm[b + k + 1] = f;
                    --k;
                }
                d.perm[b + k + 1] = e0;
            }
        }
        __syncwarp();
        for (int k = lane; k < n; k += 32) gather_one<FM>(d, g, c, __ldcg(d.perm + b + k), b + k, carry_forces);
    }
}

// Canonical order inside each cell (ascending caller index), and every atom
// moved from the scratch copy to its final slot.  One warp per cell: an
// element's rank is the number of smaller keys (keys are distinct caller
// indices), found by shuffling the cell's keys across the warp; the warp then
// gathers the cell's atoms to cell_start + rank.  A warp takes two
// neighbouring cells (work items 2w, 2w + 1) at a time: when both are in the
// same cell-mode replica and hold at most 32 atoms, their loads, ranks and
// gathers interleave, so twice the memory requests are in flight (the phase
// is latency-bound); otherwise the cells go one after the other.  Cells of
// brute-mode replicas are already in canonical (identity) order.
// carry_forces: also move frc/epot/evir (a refresh that no force evaluation
// follows).
template <bool FM>
__device__ void phase_sort_gather(const Dev& d, bool carry_forces) {
    const int N = d.ntot;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    CellGeom g;
    g.r = -1;
    const int m = __ldcg(d.rb), nwork = __ldcg(rb_cell_off(d) + m);
    for (int wp = gw; 2 * wp < nwork; wp += nw) {
        const int w0 = 2 * wp;
        const int i = rb_locate(rb_cell_off(d), m, w0);
        const int r = __ldcg(rb_rep(d) + i);
        const int off0 = __ldcg(rb_cell_off(d) + i), off1 = __ldcg(rb_cell_off(d) + i + 1);
        const int c0 = __ldcg(&d.rep[r].cell_base) + w0 - off0;
        const bool two = w0 + 1 < off1;   // the second cell is in the same replica
        const int b0 = __ldcg(d.cell_start + c0), n0 = __ldcg(d.cell_count + c0);
        const int b1 = two ? __ldcg(d.cell_start + c0 + 1) : 0, n1 = two ? __ldcg(d.cell_count + c0 + 1) : 0;
        if (r != g.r) load_geom(d, r, g);
        const bool in0 = b0 >= 0 && b0 + n0 <= N, in1 = b1 >= 0 && b1 + n1 <= N;
        if (two && g.mode == MODE_CELLS && n0 <= 32 && n1 <= 32 && in0 && in1) {
            const int e0 = lane < n0 ? __ldcg(d.perm + b0 + lane) : -1;
            const int e1 = lane < n1 ? __ldcg(d.perm + b1 + lane) : -1;
            const bool ok0 = e0 >= 0 && e0 < N, ok1 = e1 >= 0 && e1 < N;
            if ((lane < n0 && !ok0) || (lane < n1 && !ok1)) atomicOr(d.err, E_BOUNDS);
            const int key0 = ok0 ? __ldcg(d.tmp_i + e0) : 0x7FFFFFFF;
            const int key1 = ok1 ? __ldcg(d.tmp_i + e1) : 0x7FFFFFFF;
            int rank0 = 0, rank1 = 0;
            const int nm = max(n0, n1);
            for (int k = 0; k < nm; ++k) {
                rank0 += (__shfl_sync(0xffffffffu, key0, k) < key0) ? 1 : 0;
                rank1 += (__shfl_sync(0xffffffffu, key1, k) < key1) ? 1 : 0;
            }
            const bool go0 = ok0 && rank0 < n0 && gather_ok(d, g, e0, b0 + rank0);
            const bool go1 = ok1 && rank1 < n1 && gather_ok(d, g, e1, b1 + rank1);
            GatherIn g0, g1;
            if (go0) gather_load(d, e0, g0);
            if (go1) gather_load(d, e1, g1);
            if (go0) gather_store<FM>(d, g, c0, e0, b0 + rank0, g0, carry_forces);
            if (go1) gather_store<FM>(d, g, c0 + 1, e1, b1 + rank1, g1, carry_forces);
            continue;
        }
        if (n0 > 0) {
            if (in0) sort_gather_cell<FM>(d, g, c0, b0, n0, carry_forces);
            else if (lane == 0) atomicOr(d.err, E_CELLS);
        }
        if (w0 + 1 >= nwork) continue;
        // the second cell on its own (it may begin the next replica)
        int r1 = r, c1 = c0 + 1, bb = b1, nn = n1;
        if (!two) {
            r1 = __ldcg(rb_rep(d) + i + 1);
            c1 = __ldcg(&d.rep[r1].cell_base);
            bb = __ldcg(d.cell_start + c1);
            nn = __ldcg(d.cell_count + c1);
            if (r1 != g.r) load_geom(d, r1, g);
        }
        if (nn > 0) {
            if (bb >= 0 && bb + nn <= N) sort_gather_cell<FM>(d, g, c1, bb, nn, carry_forces);
            else if (lane == 0) atomicOr(d.err, E_CELLS);
        }
    }
}

// Verlet neighbour list with skin: every j (of type >= type i, the
// reference's t1 <= t2 loop, potential.rs:171-172) within rlist of i.
// Per-atom builder, used for brute-mode replicas (the whole box is one cell).
__device__ void phase_build_list(const Dev& d) {
    __shared__ int smi[32];
    const int cap = d.cap;
    for (int t = blockIdx.x; t < d.ntiles; t += gridDim.x) {
        const int4 tl = d.tiles[t];
        const RepDev& R = tile_rep(d, tl.x);
        if (!R.rebuild || R.mode == MODE_CELLS) continue;  // cell-mode replicas: k_build_list
        const float rl = (float)(R.rlist * (1.0 + 1e-5));
        const float rl2 = rl * rl;
        const int s = tl.y + threadIdx.x;
        const int tpa = R.tpa;
        int cnt = 0;
        if ((int)threadIdx.x < tl.z) {
            const float4 xi = __ldcg(d.mir + s);
            const int ti = type_of(xi);
            if (R.mode == MODE_CELLS) {
                int cx, cy, cz;
                decode_cell(d.cell[s] - R.cell_base, R.nc, cx, cy, cz);
                const float cs[3] = {(float)R.cs[0], (float)R.cs[1], (float)R.cs[2]};
                for (int dz = -1; dz <= 1; ++dz) {
                    int z = cz + dz; z = z < 0 ? z + R.nc[2] : (z >= R.nc[2] ? z - R.nc[2] : z);
                    for (int dy = -1; dy <= 1; ++dy) {
                        int y = cy + dy; y = y < 0 ? y + R.nc[1] : (y >= R.nc[1] ? y - R.nc[1] : y);
                        for (int dx = -1; dx <= 1; ++dx) {
                            int x = cx + dx; x = x < 0 ? x + R.nc[0] : (x >= R.nc[0] ? x - R.nc[0] : x);
                            const int cj = R.cell_base + (x * R.nc[1] + y) * R.nc[2] + z;
                            const uint32_t code = (uint32_t)((dx + 1) + 3 * (dy + 1) + 9 * (dz + 1));
                            const float sx = (float)dx * cs[0], sy = (float)dy * cs[1], sz = (float)dz * cs[2];
                            int jb = __ldcg(d.cell_start + cj), je = jb + __ldcg(d.cell_count + cj);
                            if (jb < R.begin || je > R.begin + R.n) { atomicOr(d.err, E_CELLS); continue; }
                            for (int j = jb; j < je; ++j) {
                                if (j == s) continue;
                                const float4 xj = __ldcg(d.mir + j);
                                if (type_of(xj) < ti) continue;
                                const float ex = xj.x - xi.x + sx, ey = xj.y - xi.y + sy,
                                            ez = xj.z - xi.z + sz;
                                if (ex * ex + ey * ey + ez * ez < rl2) {
                                    if (cnt < cap) d.nbr[list_index(s, cnt, tpa, R.begin, R.n, cap)] = (uint32_t)j | (code << IDX_BITS);
                                    ++cnt;
                                }
                            }
                        }
                    }
                }
            } else {
                const float L[3] = {(float)R.box[0], (float)R.box[1], (float)R.box[2]};
                for (int j = (int)R.begin; j < (int)R.begin + R.n; ++j) {
                    if (j == s) continue;
                    const float4 xj = __ldcg(d.mir + j);
                    if (type_of(xj) < ti) continue;
                    float e[3] = {xj.x - xi.x, xj.y - xi.y, xj.z - xi.z};
                    for (int a = 0; a < 3; ++a) {
                        if (e[a] < -0.5f * L[a]) e[a] += L[a];
                        else if (e[a] > 0.5f * L[a]) e[a] -= L[a];
                    }
                    if (e[0] * e[0] + e[1] * e[1] + e[2] * e[2] < rl2) {
                        if (cnt < cap) d.nbr[list_index(s, cnt, tpa, R.begin, R.n, cap)] = (uint32_t)j | ((uint32_t)CODE_ZERO << IDX_BITS);
                        ++cnt;
                    }
                }
            }
            const int n = min(cnt, cap);
            if (d.refmode) sort_list_by_rank(d, s, n, tpa, R.begin, R.n);
            d.nn[s] = n;
            if (cnt > cap) {
                atomicOr(d.err, E_NLIST);
                atomicMax(d.max_needed, cnt);
            }
        }
        const int bm = block_max_int(cnt, smi);
        if (threadIdx.x == 0) atomicMax(&d.rep[tl.x].max_nn, bm);
    }
}

// ---------------------------------------------------------------------------
// The per-step cooperative kernel.  Block = TILE threads.
// Phase timing for MDGB_FLAG_TRACE: block 0 stamps the time after each grid
// barrier (all blocks have finished the phase by then).
struct PhaseClock {
    unsigned long long* tr;
    unsigned long long last;
    __device__ __forceinline__ explicit PhaseClock(unsigned long long* t)
        : tr((blockIdx.x == 0 && threadIdx.x == 0) ? t : nullptr), last(0) {
        if (tr) { last = global_ns(); atomicAdd(tr + TR_LAUNCHES, 1ull); }
    }
    __device__ __forceinline__ void mark(int slot) {
        if (!tr) return;
        const unsigned long long now = global_ns();
        atomicAdd(tr + slot, now - last);
        last = now;
    }
};

__device__ __forceinline__ void k_pre_rebuild(const Dev& d, const StepParams& sp, PhaseClock& clk);

// 6 blocks of 128 threads per SM (80 registers): at the default 64 registers
// the phases spilled (measured: the rebuild's sort phases ran ~1.8x slower).
__global__ void __launch_bounds__(TILE, 6) k_pre(Dev d, StepParams sp) {
    if (chunk_failed(d)) return;
    barrier_setup(sp);
    tile_rep_reset();
    if (sp.hold_block == (int)blockIdx.x && threadIdx.x == 0) {
        // failure test: this block enters its first barrier after the others
        // have given up waiting (a bounded delay of twice the wait limit)
        const long long t0 = clock64();
        while (clock64() - t0 < 2 * g_bar_limit) __nanosleep(1000);
    }
    __syncthreads();
    PhaseClock clk(d.trace);
    if (sp.predrifted) {
        // the fused force pass of the previous step kicked and drifted (NVE
        // chunks).  Every block evaluates the rebuild test of every replica
        // (same inputs, same answer); when no replica needs one -- most
        // steps -- block 0 does the bookkeeping and all return without a
        // grid barrier.
        bool any = false;
        for (int r = threadIdx.x; r < d.nrep; r += blockDim.x) any |= rebuild_needed_at(d, sp, d.rep + r);
        if (!__syncthreads_or(any)) {
            if (blockIdx.x == 0) {
                for (int r = threadIdx.x; r < d.nrep; r += blockDim.x) {
                    RepDev* W = d.rep + r;
                    W->pending = W->baro_on ? W->myu : 1.0;
                    W->steps_since = W->steps_since + 1;
                    W->rebuild = 0;
                }
            }
            clk.mark(TR_DECIDE);
            return;
        }
        phase_decide(d, sp);
        if (grid_barrier(d)) return;
        clk.mark(TR_DECIDE);
        if (*(volatile unsigned int*)(d.bar + 2) == 0u) return;
        if (clk.tr) atomicAdd(clk.tr + TR_REBUILD_LAUNCHES, 1ull);
        k_pre_rebuild(d, sp, clk);
        return;
    }
    if (sp.do_drift && sp.coupled) {
        const int sel = d.last_type;
        // Nose-Hoover with several types: calculate_lambda runs once per type,
        // each adding its psi_dot * dt/2 (thermostat.rs:35-39, called per type
        // from integrator.rs:23-26); the last type's pass below adds its own
        // and sets lambda from the sum
        if (sp.thermo_nh)
            for (int t = 0; t < sel; ++t)
                if (nh_psi_of_type(d, sp, t)) return;
        if (d.refmode) {
            phase_serial(d, sp, sel, true);
            if (grid_barrier(d)) return;
        } else if (d.mixed && d.ntot >= FX_MIN_ATOMS) {
            phase_partials_fx(d, sel);
            if (grid_barrier(d)) return;
            phase_chunk_sums_fx(d);
            if (grid_barrier(d)) return;
            phase_finalize_fx(d, sp, sel);
            if (grid_barrier(d)) return;
        } else if (d.mixed) {
            phase_partials1(d, sel);
            if (grid_barrier(d)) return;
            phase_chunk_sums<7>(d);
            if (grid_barrier(d)) return;
            phase_finalize_single(d, sp, sel);
            if (grid_barrier(d)) return;
        } else {
            phase_partials1(d, sel);
            if (grid_barrier(d)) return;
            phase_chunk_sums<7>(d);
            if (grid_barrier(d)) return;
            phase_finalize1(d, sel);
            if (grid_barrier(d)) return;
            phase_partials2(d, sel);
            if (grid_barrier(d)) return;
            phase_chunk_sums<1>(d);
            if (grid_barrier(d)) return;
            phase_finalize2(d, sp, true, sel);
            if (grid_barrier(d)) return;
        }
        clk.mark(TR_COUPLING);
    }
    if (sp.do_drift && sp.thermo_nh) {
        if (d.mixed) phase_kick<true>(d, sp); else phase_kick<false>(d, sp);
        if (grid_barrier(d)) return;
        // Thermostat::update per type after the kick (integrator.rs:35-39):
        // each type's temperature before its scaling adds psi_dot * dt/2
        // (thermostat.rs:59-65); the scaling itself uses the lambda computed
        // before the kick, in the drift phase
        for (int t = 0; t <= d.last_type; ++t)
            if (nh_psi_of_type(d, sp, t)) return;
        if (d.mixed) phase_drift<true>(d, sp, true); else phase_drift<false>(d, sp, true);
        if (grid_barrier(d)) return;
    } else if (sp.do_drift || !sp.force_rebuild) {
        // (a forced rebuild without a step -- upload, refresh -- recomputes
        // every mirror in its gather: nothing here to do for it)
        if (d.mixed) phase_drift<true>(d, sp, false); else phase_drift<false>(d, sp, false);
        if (grid_barrier(d)) return;
    }
    clk.mark(TR_DRIFT);
    phase_decide(d, sp);
    if (grid_barrier(d)) return;
    clk.mark(TR_DECIDE);
    if (*(volatile unsigned int*)(d.bar + 2) == 0u) return;
    if (clk.tr) atomicAdd(clk.tr + TR_REBUILD_LAUNCHES, 1ull);
    k_pre_rebuild(d, sp, clk);
}

// The rebuild phases of k_pre (replicas with their rebuild flag set).
__device__ __forceinline__ void k_pre_rebuild(const Dev& d, const StepParams& sp, PhaseClock& clk) {
    if (blockIdx.x == 0) phase_work_list(d);
    phase_zero_cells(d);
    if (grid_barrier(d)) return;
    clk.mark(TR_ZERO);
    phase_bin(d);
    if (grid_barrier(d)) return;
    clk.mark(TR_BIN);
    const int chunk = (d.ncells + gridDim.x - 1) / gridDim.x;
    phase_scan_a(d, chunk);
    if (grid_barrier(d)) return;
    clk.mark(TR_SCAN_A);
    phase_scan_b(d);
    if (grid_barrier(d)) return;
    clk.mark(TR_SCAN_B);
    phase_scan_c(d, chunk);
    if (grid_barrier(d)) return;
    clk.mark(TR_SCAN_C);
    phase_scatter(d, !sp.do_drift);
    if (grid_barrier(d)) return;
    clk.mark(TR_SCATTER);
    if (d.mixed) phase_sort_gather<true>(d, !sp.do_drift); else phase_sort_gather<false>(d, !sp.do_drift);
    if (grid_barrier(d)) return;
    clk.mark(TR_GATHER);
    if (clk.tr) clk.tr[TR_STAMP] = clk.last;
    // brute-mode replicas here; cell-mode replicas in k_build_list, which
    // follows this kernel and closes the rebuild
    phase_build_list(d);
}

// Macro parameters of type `sel` (solver/src/macro_parameters): results land
// in the replica records (vcm, mom, ke, pe, thermal, T, P, count).
__global__ void __launch_bounds__(TILE) k_macro(Dev d, StepParams sp, int sel) {
    barrier_setup(sp);
    tile_rep_reset();
    if (d.refmode) {
        phase_serial(d, sp, sel, false);
        return;
    }
    phase_partials1(d, sel);
    if (grid_barrier(d)) return;
    phase_chunk_sums<7>(d);
    if (grid_barrier(d)) return;
    phase_finalize1(d, sel);
    if (grid_barrier(d)) return;
    phase_partials2(d, sel);
    if (grid_barrier(d)) return;
    phase_chunk_sums<1>(d);
    if (grid_barrier(d)) return;
    phase_finalize2(d, sp, false, sel);
}

// End of an mdgb_step call: finish the barostat update of the last step
// (x *= mu; the box part was applied... here as well, once per type).
__global__ void __launch_bounds__(TILE) k_apply_pending(Dev d) {
    const int t = blockIdx.x;
    if (t >= d.ntiles) return;
    const int4 tl = d.tiles[t];
    const double f = d.rep[tl.x].pending;
    if (f == 1.0) return;
    const int s = tl.y + threadIdx.x;
    if ((int)threadIdx.x < tl.z) {
        double4_32a p = d.pos[s];
        p.x = __dmul_rn(p.x, f); p.y = __dmul_rn(p.y, f); p.z = __dmul_rn(p.z, f);
        d.pos[s] = p;
    }
}

__global__ void k_apply_pending_box(Dev d) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= d.nrep) return;
    RepDev* W = d.rep + r;
    const double f = W->pending;
    if (f == 1.0) return;
    for (int k = 0; k < d.ntypes; ++k)
        for (int a = 0; a < 3; ++a) W->box[a] *= f;
    for (int a = 0; a < 3; ++a) W->cs[a] = W->box[a] / (double)W->nc[a];
    W->pending = 1.0;
}

// Device -> caller order (for download): out[orig[s]] = value[s]; a null
// output is skipped.
__global__ void k_gather_out(Dev d, double* out_pos, double* out_vel, double* out_frc,
                             double* out_pot, double* out_tmp) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.ntot;
    if (s >= N) return;
    const int o = d.orig[s];
    if (o < 0 || o >= N) { atomicOr(d.err, E_BOUNDS); return; }
    if (out_pos) {
        const double4_32a p = d.pos[s];
        out_pos[3 * (size_t)o] = p.x; out_pos[3 * (size_t)o + 1] = p.y; out_pos[3 * (size_t)o + 2] = p.z;
    }
    for (int k = 0; k < 3; ++k) {
        if (out_vel) out_vel[3 * (size_t)o + k] = d.vel[(size_t)k * N + s];
        if (out_frc) out_frc[3 * (size_t)o + k] = d.frc[(size_t)k * N + s];
    }
    if (out_pot) out_pot[o] = d.epot[s];
    if (out_tmp) out_tmp[o] = d.evir[s];
}

// Caller order -> device (upload): the device order starts as the caller's;
// the first rebuild sorts it by cell.  in_rank null: one type, the rank is the
// index.  A type id >= ntypes is flagged (E_INPUT) and replaced by 0, so no
// later kernel indexes the pair table with it.
__global__ void k_scatter_in(Dev d, const double* in_pos, const double* in_vel, const uint16_t* in_type,
                             const int* in_rank, int ntypes) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.ntot;
    if (s >= N) return;
    int ty = (int)in_type[s];
    if (ty >= ntypes) { atomicOr(d.err, E_INPUT); ty = 0; }
    double4_32a p;
    p.x = in_pos[3 * (size_t)s]; p.y = in_pos[3 * (size_t)s + 1]; p.z = in_pos[3 * (size_t)s + 2];
    p.w = __longlong_as_double((long long)ty);
    d.pos[s] = p;
    for (int k = 0; k < 3; ++k) {
        d.vel[(size_t)k * N + s] = in_vel ? in_vel[3 * (size_t)s + k] : 0.0;
        d.frc[(size_t)k * N + s] = 0.0;
    }
    d.epot[s] = 0.0;
    d.evir[s] = 0.0;
    d.orig[s] = s;
    int rk = in_rank ? in_rank[s] : s;
    if (rk < 0 || rk >= N) { atomicOr(d.err, E_BOUNDS); rk = s; }
    d.rank[s] = rk;
    d.slot_of_rank[rk] = s;
    d.cell[s] = -1;
    d.nn[s] = 0;
    d.mir0[s] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Caller order -> device order for force, potential, temp (mdgb_upload_forces).
__global__ void k_scatter_forces(Dev d, const double* in_frc, const double* in_pot, const double* in_tmp) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.ntot;
    if (s >= N) return;
    const int o = d.orig[s];
    if (o < 0 || o >= N) { atomicOr(d.err, E_BOUNDS); return; }
    if (in_frc)
        for (int k = 0; k < 3; ++k) d.frc[(size_t)k * N + s] = in_frc[3 * (size_t)o + k];
    if (in_pot) d.epot[s] = in_pot[o];
    if (in_tmp) d.evir[s] = in_tmp[o];
}

// Interacting pairs from the neighbour list, decided with the reference's
// FP64 arithmetic (potential.rs:181-204), in caller indices.
__global__ void k_pairs(Dev d, long long capacity, int* out_i, int* out_j, unsigned long long* count) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = d.ntot;
    if (s >= N) return;
    int r = 0;
    {
        // replica of s: tiles are contiguous per replica
        int lo = 0, hi = d.nrep - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (d.rep[mid].begin <= s) lo = mid; else hi = mid - 1;
        }
        r = lo;
    }
    const RepDev& R = d.rep[r];
    const double4_32a pi = d.pos[s];
    const int ti = type_of(pi);
    const int n = d.nn[s];
    for (int k = 0; k < n; ++k) {
        const uint32_t e = d.nbr[list_index(s, k, R.tpa, R.begin, R.n, d.cap)];
        const int j = (int)(e & IDX_MASK);
        if (j < 0 || j >= N) { atomicOr(d.err, E_BOUNDS); continue; }
        const double4_32a pj = d.pos[j];
        const PairDev& P = d.pair[ti * MAX_TYPES + type_of(pj)];
        double rx = pj.x - pi.x, ry = pj.y - pi.y, rz = pj.z - pi.z;
        if (rx < -(R.box[0] / 2.0)) rx += R.box[0]; else if (rx > R.box[0] / 2.0) rx -= R.box[0];
        if (ry < -(R.box[1] / 2.0)) ry += R.box[1]; else if (ry > R.box[1] / 2.0) ry -= R.box[1];
        if (rz < -(R.box[2] / 2.0)) rz += R.box[2]; else if (rz > R.box[2] / 2.0) rz -= R.box[2];
        const double ra = sqrt(rx * rx + ry * ry + rz * rz);
        if (ra > P.rc) continue;
        const unsigned long long slot = atomicAdd(count, 1ull);
        if ((long long)slot < capacity) {
            out_i[slot] = d.orig[s];
            out_j[slot] = d.orig[j];
        }
    }
}

}  // namespace mdgb
