// mdgb_internal.cuh -- device data layout of the GB300 MD step engine.
//
// One engine holds R >= 1 independent replicas (a single system is R = 1).
// Atoms of replica r occupy the contiguous device range [begin_r, begin_r+n_r)
// and are kept sorted by cell (counting sort at every list rebuild), so the
// atoms a tile reads as neighbours sit close together in HBM/L2.  All
// per-atom work is organised in tiles of TILE atoms that never straddle a
// replica; kernels take tiles as their unit of work.
//
// HBM layout, per atom (sorted order):
//   pos   double4_32a  FP64 master position, .w carries the type id bits
//   vel   double   SoA [3][N]
//   frc   double   SoA [3][N]       force of the last evaluation
//   epot  double   [N]              the reference's Particle::potential
//   evir  double   [N]              the reference's Particle::temp (sum of f.r)
//   mir   float4   FP32 mirror: position relative to the centre of the atom's
//                  (frozen) cell, .w = type bits -- the mixed path's gather
//   mir0  float4   mirror at the last rebuild (displacement check)
//   cell  int      frozen cell (global index)
//   orig  int      index of the atom in the caller's flat array
//   rank  int      reference order: type-major index (particles[t][k])
//   nn    int      neighbour count;  nbr uint32 [cap][N] (tpa-interleaved)
//   lmask uint32   [27][N] the paired list build's hit words (rebuild scratch)
// A neighbour entry is (j | code << 27): j the sorted index, code in 0..26
// the periodic cell shift (dx,dy,dz in -1..1) used by the mixed path.
// Per cell: count, start, the tagged starts of its 27 neighbour cells (nbs);
// per rebuild: the work list of rebuilding replicas (rb).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mdgb {

constexpr int MAX_TYPES = 16;
constexpr int TILE = 128;
constexpr int IDX_BITS = 27;
constexpr uint32_t IDX_MASK = (1u << IDX_BITS) - 1u;
constexpr int CODE_ZERO = 13;  // (0,0,0)
constexpr int CHUNK_TILES = 256;  // tiles per reduction chunk

// error bits (device word, read by the host after each chunk)
enum : int {
    E_NLIST = 1,      // neighbour list capacity exceeded
    E_TIMEOUT = 2,    // a bounded grid-barrier wait gave up
    E_FIXED = 4,      // fixed-point force accumulator out of range
    E_SKIN = 8,       // fixed rebuild interval let an atom move too far
    E_BOUNDS = 16,    // an index derived from scratch data was out of range
    E_CELLS = 32,     // cell bookkeeping inconsistent
    E_INPUT = 64,     // an uploaded type id >= ntypes
};

enum : int { MODE_CELLS = 0, MODE_BRUTE = 1 };

// Pair potential (Lennard-Jones, potential.rs:12-18).  FP64 fields are the
// reference's values; FP32 fields feed the mixed path.
struct PairDev {
    double sigma, eps, rc, ucut, eps4, eps24;
    float sig2f, eps4f, eps24f, ucutf;
    float rc2f_lo, rc2f_hi;  // band around rc^2 decided exactly in FP64
    int pad0, pad1;
    double rc2_cut;          // smallest double whose rounded square root exceeds rc
};

struct RepDev {
    // static, set at upload
    long long begin;
    int n, cell_base, cell_cap, tile_begin, ntiles, last_type_count;
    int chunk_begin, nchunks;     // reduction chunks of <= CHUNK_TILES tiles
    int tpa;                      // threads per atom of this replica's size class (list layout)
    int size_class;
    int type_off[MAX_TYPES + 1];  // reference order: type t owns ranks [begin+off[t], begin+off[t+1])
    // geometry (device-updated)
    double box[3];
    double box_build[3];
    double cs[3];
    double inv_cs[3];             // nc / box at the rebuild (binning)
    int nc[3];
    int mode;
    // coupling
    int thermo_on, thermo_kind, baro_on, pad0;
    double th_tau, th_T0, lambda, psi;
    double ba_beta, ba_tau, ba_P0, myu;
    double pending;        // barostat factor still to apply to positions (1 = none)
    double rlist;          // list radius: the largest r_cut + this replica's skin (its size class's)
    // rebuild bookkeeping
    unsigned int max_disp_bits;
    int rebuild;
    int steps_since;
    int nrebuilds;
    int max_nn;
    int pad1;
    // reductions (coupling or macro)
    double vcm[3], msum, thermal, ke, pe, virsum, T, P, mom[3];
    long long count;
};

// One row of the exact (128-bit fixed-point) sums of the mixed path's coupled
// steps: per quantity (v_x, v_y, v_z, temp, v.v, potential) an integer sum on
// the binary grid of its exponent ex (unit 2^(ex - 1075 - FX_K)), the atom
// count and a flag for non-finite inputs.  128 bytes.
constexpr int FX_NQ = 6;
constexpr int FX_K = 44;
struct __align__(16) FxRow {
    __int128 s[FX_NQ];
    unsigned short ex[FX_NQ];
    int nonfinite;
    long long count;
};
static_assert(sizeof(FxRow) == 128, "FxRow is 128 bytes");

struct StepParams {
    double dt;
    double kick_c[MAX_TYPES];  // dt / (2 m_t), computed on the host as the reference does
    int coupled;               // any thermostat/barostat active
    int thermo_nh;             // Nose-Hoover present (two-stage update)
    int fixed_interval;        // >0: rebuild every that many steps
    int force_rebuild;         // rebuild every replica now
    int do_drift;              // 0: only (re)build / refresh, no integration
    int predrifted;            // the previous force pass already kicked and drifted (NVE)
    int fused;                 // force pass: also the next step's kick and drift (into pos_next/mir_next)
    int hold_block;            // >= 0: that block of the step kernel enters its first grid barrier late
                               //   (failure test of the bounded barrier; -1 in every normal step)
    long long barrier_cycles;  // > 0: the grid barrier's wait limit in clock cycles (0: the default, ~2 s)
};

// Everything a kernel needs, passed by value.
struct Dev {
    int ntot, ntiles, nrep, ntypes, cap, tpa, ncells;
    int refmode, mixed, single_type, last_type, direct_list;   // direct_list: MDGB_FLAG_DIRECT_LIST
    double mass[MAX_TYPES];
    double rlist, rcmax, skin;   // rlist: the largest list radius of any replica
    float fscale, inv_fscale_f;  // fixed-point scale 2^fscale_log2
    double inv_fscale;
    int fscale_log2, pad_fs;
    double4_32a* pos;
    double* vel;
    double* frc;
    double* epot;
    double* evir;
    float4* mir;
    float4* mir0;
    int* cell;
    int* orig;
    int* rank;
    int* nn;
    uint32_t* nbr;
    int4* tiles;       // (replica, begin, count, 0)
    RepDev* rep;
    const PairDev* pair;  // [MAX_TYPES*MAX_TYPES]
    double* part;      // [ntiles][8] tile partials
    double* cpart;     // [nchunks][8] chunk partials
    int4* chunks;      // (replica, first tile, tile count, 0)
    int nchunks, pad_ch;
    int* err;
    int* max_needed;   // largest neighbour count requested
    // rebuild scratch
    int* cell_count;
    int* cell_start;   // [ncells+1]
    int* cell_rep;     // replica of each cell
    int* perm;
    double4_32a* tmp_pos;
    double* tmp_d;     // [8][N]: vel3, frc3, epot, evir
    int* tmp_i;        // [4][N]: orig, rank, cell, slot within the cell
    int* slot_of_rank;
    int* bsum;         // [grid] scan block sums
    unsigned int* bar; // [8] grid barrier count, generation; any rebuild; list-build blocks done;
                       //   a cell too crowded for the paired list build; direct builds so far
    int* rb;           // rebuild work list, built by the step kernel when it rebuilds:
                       //   [0] count m of rebuilding replicas, [1] how many of them come
                       //   first because the paired list build does not take them (brute
                       //   mode, or fewer than LIST_PAIRED_MIN_ATOMS atoms), then nrep ids,
                       //   m + 1 prefix offsets of their cells and m + 1 of their tiles
    uint32_t* lmask;   // [27][N] paired list build: hit word of (shift code, atom)
    uint32_t* nbs;     // [ncells][27] start of each neighbour cell, tagged with its shift code
    unsigned int* queue;  // persistent force kernel work counters (one per size class)
    int* tile_order;   // tiles grouped by size class, costliest first inside a class
    const int* tile_list;  // the tiles one force launch covers (a size class)
    int ntile_list, list_class;
    unsigned long long* trace;  // MDGB_FLAG_TRACE: per-phase nanoseconds of k_pre (else null)
    double4_32a* pos_next;      // fused drift: where the force kernel writes the next positions
    float4* mir_next;           //   and mirrors (the other buffer of each pair)
    int2* band_list;            // mixed path: atoms (index, replica) left to k_force_band
    int* band_count;
    FxRow* fx_part;             // [ntiles] exact tile sums (mixed path, coupled steps)
    FxRow* fx_cpart;            // [nchunks] exact chunk sums
};

// k_pre phases recorded with MDGB_FLAG_TRACE (slot indices; TR_SORT stays 0,
// the in-cell sort is part of the gather phase)
enum : int {
    TR_COUPLING = 0, TR_DRIFT, TR_DECIDE, TR_ZERO, TR_BIN, TR_SCAN_A, TR_SCAN_B, TR_SCAN_C,
    TR_SCATTER, TR_SORT, TR_GATHER, TR_LIST, TR_LAUNCHES, TR_REBUILD_LAUNCHES,
    TR_STAMP = 15,   // time stamp the list-build kernel measures from
    TR_SLOTS = 16
};

// A failed grid barrier earlier in this chunk (E_TIMEOUT): the launches that
// follow in the chunk do nothing (the engine restores the chunk's starting
// state and reports MDGB_ERR_DEVICE_TIMEOUT).
__device__ __forceinline__ bool chunk_failed(const Dev& d) {
    return (*(volatile const int*)d.err & E_TIMEOUT) != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The rebuild work list (Dev::rb): replica ids and prefix offsets of their
// cells and tiles.  Work item w (a cell or a tile of a rebuilding replica,
// counted over the list) -> the list position i with off[i] <= w < off[i+1].
constexpr int LIST_PAIRED_MIN_ATOMS = 32768;  // smaller replicas: the direct list build
__device__ __forceinline__ const int* rb_rep(const Dev& d) { return d.rb + 2; }
__device__ __forceinline__ const int* rb_cell_off(const Dev& d) { return d.rb + 2 + d.nrep; }
__device__ __forceinline__ const int* rb_tile_off(const Dev& d) { return d.rb + 3 + 2 * d.nrep; }
__device__ __forceinline__ int rb_locate(const int* off, int m, int w) {
    int lo = 0, hi = m - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldcg(off + mid) <= w) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Verlet-list build for cell-mode replicas (kernels_list.cu): a kernel that
// follows every k_pre launch and closes the rebuild k_pre started.
cudaError_t list_build_init();
int list_build_grid(const Dev& d, int num_sms);
int list_masks_grid(const Dev& d, int num_sms);
cudaError_t launch_list_build(const Dev& d, int grid, int mgrid, cudaStream_t st);

__device__ __forceinline__ int type_of(double4_32a p) { return (int)__double_as_longlong(p.w); }
__device__ __forceinline__ int type_of(float4 p) { return __float_as_int(p.w); }

// IEEE-754 format conversions with integer operations (GB300's float<->double
// conversion instructions issue on its narrow FP64 pipe).  Written from the
// binary formats: exponent rebias 1023 <-> 127, mantissa 52 <-> 23 bits.
//
// double -> float, round to nearest even, for |x| in [2^-126, 2^128); smaller
// magnitudes give +-0 (the engine only converts bounded, well-scaled values).
__device__ __forceinline__ float dbl_to_flt_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long mag = b & 0x7FFFFFFFFFFFFFFFull;
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    if (mag < 0x3810000000000000ull) return __uint_as_float(sign);  // below 2^-126
    unsigned long long r = mag >> 29;
    const unsigned rem = (unsigned)(mag & 0x1FFFFFFFull);
    r += (rem > 0x10000000u) | ((rem == 0x10000000u) & (unsigned)(r & 1ull));
    return __uint_as_float((unsigned)(r - (896ull << 23)) | sign);
}

// float -> double (exact) for normal floats and zero.
__device__ __forceinline__ double flt_to_dbl(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned mag = u & 0x7FFFFFFFu;
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    if (mag == 0u) return __longlong_as_double((long long)sign);
    return __longlong_as_double((long long)((((unsigned long long)mag << 29) + (896ull << 52)) | sign));
}

// Two floats in one 64-bit register pair (lo, hi) for GB300's paired FP32
// instructions (add/sub/mul/fma .f32x2: two IEEE round-to-nearest operations
// per instruction).
typedef unsigned long long f2_t;
__device__ __forceinline__ f2_t f2(float lo, float hi) {
    f2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float f2_lo(f2_t v) { return __uint_as_float((unsigned)v); }
__device__ __forceinline__ float f2_hi(f2_t v) { return __uint_as_float((unsigned)(v >> 32)); }
__device__ __forceinline__ f2_t add2(f2_t a, f2_t b) {
    f2_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t sub2(f2_t a, f2_t b) {
    f2_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t mul2(f2_t a, f2_t b) {
    f2_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t fma2(f2_t a, f2_t b, f2_t c) {
    f2_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Exact int64 -> double for |x| < 2^53 with integer operations (the top bit
// found with a count of leading zeros, the mantissa shifted into place), then
// scaled by 2^-k through the exponent (k small enough that the result stays a
// normal number); larger |x| take the rounding conversion instruction.
__device__ __forceinline__ double fixed_to_double(long long x, int k) {
    if (x == 0) return 0.0;
    const unsigned long long sign = x < 0 ? 0x8000000000000000ull : 0ull;
    const unsigned long long m = x < 0 ? 0ull - (unsigned long long)x : (unsigned long long)x;
    if (m >= (1ull << 53))
        return __longlong_as_double(__double_as_longlong(__ll2double_rn(x)) - ((long long)k << 52));
    const int lz = __clzll((long long)m);   // >= 11
    const unsigned long long mant = (m << (lz - 11)) & 0x000FFFFFFFFFFFFFull;
    const unsigned long long ex = (unsigned long long)(63 - lz + 1023 - k);
    return __longlong_as_double((long long)(sign | (ex << 52) | mant));
}

// Neighbour entry k of atom s.  Replica r owns the list segment starting at
// cap * begin_r, laid out [k / tpa][atom][k % tpa] with its own threads per
// atom, so the tpa lanes of one atom read consecutive words and consecutive
// atoms of a warp read consecutive groups (coalesced for every tpa).
__host__ __device__ __forceinline__ size_t list_index(int s, int k, int tpa, long long begin, int n, int cap) {
    return (size_t)cap * (size_t)begin +
           ((size_t)(k / tpa) * (size_t)n + (size_t)(s - begin)) * (size_t)tpa + (size_t)(k % tpa);
}

__device__ __forceinline__ void decode_cell(int l, const int nc[3], int& cx, int& cy, int& cz) {
    cz = l % nc[2];
    const int q = l / nc[2];
    cy = q % nc[1];
    cx = q / nc[1];
}

// ---------------------------------------------------------------------------
// Drift arithmetic shared by the step kernel and the force kernel's fused
// drift; every operation is an explicit round-to-nearest intrinsic, so both
// translation units (compiled with different contraction settings) produce
// the same bits.

// x + y and x * y rounded to nearest, for operations under a branch that is
// rarely or conditionally taken: as volatile inline PTX the compiler cannot
// evaluate them unconditionally and select the result (which it does with
// __dadd_rn / __dmul_rn, costing FP64 operations on every call on GB300's
// narrow FP64 pipe).  Same bits as __dadd_rn / __dmul_rn.
__device__ __forceinline__ double dadd_nospec(double x, double y) {
    double r;
    asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(x), "d"(y));
    return r;
}
__device__ __forceinline__ double dmul_nospec(double x, double y) {
    double r;
    asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(x), "d"(y));
    return r;
}

// core/src/particle.rs:120-141 with the comparisons done on the bit patterns:
// for x >= 0 and L > 0 the signed 64-bit order of the bits is the numeric
// order, and x < 0.0 is "sign bit set and not -0.0".  x - L is x + (-L).
__device__ __forceinline__ double wrap_ref(double x, double L) {
    const long long b = __double_as_longlong(x);
    if (b < 0 && b != (long long)0x8000000000000000ull) return dadd_nospec(x, L);
    if (b >= __double_as_longlong(L)) return dadd_nospec(x, -L);
    return x;
}

// a + b * c: the reference's two roundings (FP64 path) or one fused
// multiply-add (mixed path: half the operations on GB300's narrow FP64 pipe).
// `fused` must be a compile-time constant at every call (a run-time flag has
// the compiler evaluate both forms and select).
__device__ __forceinline__ double madd(double a, double b, double c, bool fused) {
    return fused ? __fma_rn(b, c, a) : __dadd_rn(a, __dmul_rn(b, c));
}

// integrator.rs:42-46 drift x += v dt, then a single periodic shift per axis.
__device__ __forceinline__ double4_32a drift_wrap(double4_32a p, double vx, double vy, double vz, double dt,
                                                  const double* box, bool fused) {
    p.x = wrap_ref(madd(p.x, vx, dt, fused), box[0]);
    p.y = wrap_ref(madd(p.y, vy, dt, fused), box[1]);
    p.z = wrap_ref(madd(p.z, vz, dt, fused), box[2]);
    return p;
}

// FP32 mirror: position relative to the centre of the atom's frozen cell,
// taken to the nearest periodic image (continuous while the atom stays near
// its cell; in brute mode the "cell" is the whole box, so it is the wrapped
// position relative to the box centre).  hL: half box in FP32.
// G: a replica record or anything else with its nc, cs and box.
template <class G>
__device__ __forceinline__ float4 mirror_of(double4_32a p, int cell_local, const G& R, const float* hL,
                                            bool fused) {
    int cx, cy, cz;
    decode_cell(cell_local, R.nc, cx, cy, cz);
    // cell centre (c + 0.5) * cs; c + 0.5 is exact in FP32 and converts exactly
    const double k[3] = {flt_to_dbl(-((float)cx + 0.5f)), flt_to_dbl(-((float)cy + 0.5f)),
                         flt_to_dbl(-((float)cz + 0.5f))};
    const double x[3] = {p.x, p.y, p.z};
    float o[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double u = madd(x[a], k[a], R.cs[a], fused);
        float f = dbl_to_flt_rn(u);
        const float h = hL[a];
        // nearest image of the atom relative to its cell centre; only atoms that
        // just crossed the periodic boundary (|u| ~ L) take this branch, far
        // from the +-L/2 decision edge, so the FP32 comparison decides it
        if (f >= h) { u = dadd_nospec(u, -R.box[a]); f = dbl_to_flt_rn(u); }
        else if (f < -h) { u = dadd_nospec(u, R.box[a]); f = dbl_to_flt_rn(u); }
        o[a] = f;
    }
    return make_float4(o[0], o[1], o[2], __int_as_float(type_of(p)));
}

// Per-replica constants of the displacement check: box (FP32), half box, and
// the box scale since the last rebuild.
__device__ __forceinline__ void drift_consts(const RepDev& R, float* tc) {
    for (int a = 0; a < 3; ++a) {
        tc[a] = dbl_to_flt_rn(R.box[a]);
        tc[3 + a] = __fmul_rn(0.5f, tc[a]);
    }
    tc[6] = dbl_to_flt_rn(__ddiv_rn(R.box[0], R.box_build[0]));
}

// Distance moved since the last rebuild (mirror against the rebuild mirror
// scaled with the box), nearest image.
__device__ __forceinline__ float mirror_disp(float4 m, float4 m0, const float* tc) {
    const float sc = tc[6];
    float dd[3] = {__fsub_rn(m.x, __fmul_rn(sc, m0.x)), __fsub_rn(m.y, __fmul_rn(sc, m0.y)),
                   __fsub_rn(m.z, __fmul_rn(sc, m0.z))};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (dd[a] > tc[3 + a]) dd[a] = __fsub_rn(dd[a], tc[a]);
        else if (dd[a] < -tc[3 + a]) dd[a] = __fadd_rn(dd[a], tc[a]);
    }
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dd[0], dd[0]), __fmul_rn(dd[1], dd[1])),
                                __fmul_rn(dd[2], dd[2])));
}

// A replica record read through L2 (other blocks may have written it in
// this launch).
__device__ __forceinline__ RepDev load_rep(const RepDev* p) {
    RepDev r;
    const long long* src = reinterpret_cast<const long long*>(p);
    long long* dst = reinterpret_cast<long long*>(&r);
#pragma unroll 4
    for (int i = 0; i < (int)(sizeof(RepDev) / 8); ++i) dst[i] = __ldcg(src + i);
    return r;
}

// Per replica: consume the pending barostat factor, decide on a rebuild (and
// the new cell grid).  A pair outside the list at the rebuild had r0 >= rlist;
// after a box scale sc and displacements <= maxd it is at >= sc*rlist -
// 2*maxd, which must stay above the largest cutoff.  Explicit FP64
// intrinsics: the step kernel and the fused force pass decide alike.
__device__ __forceinline__ bool rebuild_needed(const Dev& d, const StepParams& sp, int steps_since0, int rebuild,
                                               double box0, double box_build0, unsigned max_disp_bits,
                                               double rlist) {
    const int steps_since = steps_since0 + (sp.do_drift ? 1 : 0);
    const double sc = __ddiv_rn(box0, box_build0);
    const double maxd = (double)__uint_as_float(max_disp_bits);
    const double limit = __dsub_rn(__dsub_rn(__dmul_rn(sc, rlist), d.rcmax), __dmul_rn(1e-5, rlist));
    return sp.force_rebuild || rebuild || (__dmul_rn(2.0, maxd) > limit) ||
           (sp.fixed_interval > 0 && steps_since >= sp.fixed_interval);
}
__device__ __forceinline__ bool rebuild_needed(const Dev& d, const StepParams& sp, const RepDev& R) {
    return rebuild_needed(d, sp, R.steps_since, R.rebuild, R.box[0], R.box_build[0], R.max_disp_bits, R.rlist);
}
// the same test reading only the fields it needs (through L2)
__device__ __forceinline__ bool rebuild_needed_at(const Dev& d, const StepParams& sp, const RepDev* p) {
    return rebuild_needed(d, sp, __ldcg(&p->steps_since), __ldcg(&p->rebuild), __ldcg(&p->box[0]),
                          __ldcg(&p->box_build[0]), __ldcg(&p->max_disp_bits), __ldcg(&p->rlist));
}

__device__ __forceinline__ void decide_replica(const Dev& d, const StepParams& sp, int r) {
    const RepDev R = load_rep(d.rep + r);
    RepDev* W = d.rep + r;
    int steps_since = R.steps_since;
    if (sp.do_drift) {
        W->pending = R.baro_on ? R.myu : 1.0;
        ++steps_since;
    }
    const bool need = rebuild_needed(d, sp, R);
    if (need) {
        long long nc[3];
        bool brute = R.cell_cap < 27;
        const double cmin = __dmul_rn(R.rlist, 1.0 + 1e-6);
        for (int a = 0; a < 3; ++a) {
            nc[a] = (long long)floor(__ddiv_rn(R.box[a], cmin));
            if (nc[a] < 3) brute = true;
        }
        if (!brute) {
            while (nc[0] * nc[1] * nc[2] > (long long)R.cell_cap) {
                int a = 0;
                if (nc[1] > nc[a]) a = 1;
                if (nc[2] > nc[a]) a = 2;
                --nc[a];
            }
            if (nc[0] < 3 || nc[1] < 3 || nc[2] < 3) brute = true;
        }
        if (brute) nc[0] = nc[1] = nc[2] = 1;
        for (int a = 0; a < 3; ++a) {
            W->nc[a] = (int)nc[a];
            W->cs[a] = __ddiv_rn(R.box[a], (double)nc[a]);
            W->inv_cs[a] = __ddiv_rn((double)nc[a], R.box[a]);
            W->box_build[a] = R.box[a];
        }
        W->mode = brute ? MODE_BRUTE : MODE_CELLS;
        W->max_disp_bits = 0u;
        W->max_nn = 0;
        steps_since = 0;
        W->rebuild = 1;
        atomicAdd(d.bar + 2, 1u);
    } else {
        W->rebuild = 0;
    }
    W->steps_since = steps_since;
}

// In the reference's order (refmode): ascending (type, index in type), i.e. rank.
__device__ __forceinline__ void sort_list_by_rank(const Dev& d, int s, int n, int tpa, long long begin, int nr) {
    const int cap = d.cap;
    for (int a = 1; a < n; ++a) {
        const uint32_t e = d.nbr[list_index(s, a, tpa, begin, nr, cap)];
        const int key = __ldcg(d.rank + (e & IDX_MASK));
        int k = a - 1;
        while (k >= 0) {
            const uint32_t f = d.nbr[list_index(s, k, tpa, begin, nr, cap)];
            if (__ldcg(d.rank + (f & IDX_MASK)) <= key) break;
            d.nbr[list_index(s, k + 1, tpa, begin, nr, cap)] = f;
            --k;
        }
        d.nbr[list_index(s, k + 1, tpa, begin, nr, cap)] = e;
    }
}

}  // namespace mdgb
