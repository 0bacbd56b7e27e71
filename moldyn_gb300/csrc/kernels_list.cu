// kernels_list.cu -- Verlet-list build for cell-mode replicas.
//
// Launched right after the step kernel; both kernels return at once unless
// that kernel flagged a rebuild (its binning, counting sort and gather have
// then left the atoms sorted by cell with fresh FP32 mirrors).
//
// A list is the concatenation, in shift-code order (dz outer, dx inner) and
// in cell order inside each cell, of the atoms of the 27 neighbour cells that
// lie within the replica's rlist (1 + 1e-5) in FP32 -- a superset of the
// pairs inside rlist, which the force kernels decide exactly.  Two builds
// produce it:
//
// Paired (replicas of at least LIST_PAIRED_MIN_ATOMS atoms whose cells hold
// at most 32 atoms, the usual case).  k_list_masks: one
// warp per cell A tests A's atoms against the atoms of A and of its 13
// forward neighbour cells (codes 14..26), so each pair of neighbouring cells
// is tested once, from one side.  A candidate stream of those cells is
// walked 32 candidates at a time, one per lane, each tested against every
// own atom, which gives per lane a 32-bit mask over A's atoms.  That mask is
// already the forward atom's hit row for the opposite code 26 - k; its 32x32
// bit transpose across the warp gives A's rows over the stream, cut into one
// word per code.  The words go to lmask[code][atom] (bit p: the neighbour
// cell's atom at cell_start + p); each (atom, code) word is written exactly
// once.  k_build_list then expands every atom's 27 words, lane = atom, in
// code and bit order: all lanes append entry t of their atoms in the same
// pass, so in the [k / tpa][atom][k % tpa] layout the stores of a pass are
// contiguous.
//
// Direct (smaller replicas, where the second pass costs more than the
// halved tests save; every replica when a cell of more than 32 atoms is
// anywhere in the rebuild, or with MDGB_FLAG_DIRECT_LIST).  One warp per
// cell, 32 of the cell's atoms at a
// time ("own" atoms, staged in shared memory), tests the stream of all 27
// neighbour cells, collects per lane a mask over the own atoms, transposes it
// and expands each own atom's masks into its list.
//
// Both give the same entries in the same order; the paired build decides a
// pair with one rounding of its FP32 distance, so a pair within rounding of
// rlist (1 + 1e-5) -- far outside r_cut -- is listed on both sides or on
// neither, where the direct build decides each side on its own.
#include <algorithm>

#include "mdgb_internal.cuh"

namespace mdgb {

constexpr int LB_WARPS = 2;           // warps per block
constexpr int LB_WIN = 1024;          // candidate stream positions held per window
constexpr int LB_MQ = LB_WIN / 32 + 1;  // mask row stride (odd: conflict-free columns)

// Per-warp shared memory in 32-bit words: candidate window, hit masks
// [own atom][chunk], own atoms (paired coordinates and types: 4 words each),
// the 27 cell shifts (float4).
constexpr int LB_WARP_WORDS = LB_WIN + 32 * LB_MQ + 32 * 4 + 27 * 4 + 4;
static_assert((LB_WIN + 32 * LB_MQ) % 4 == 0 && LB_WARP_WORDS % 4 == 0, "float4 alignment");

// Bit-matrix transpose over a warp: lane l holds row l (bit c = entry (l, c));
// afterwards lane c holds column c (bit l = entry (l, c)).  Five butterfly
// stages; stage j swaps the off-diagonal j x j blocks of every 2j x 2j block.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, int lane) {
    const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int st = 0; st < 5; ++st) {
        const int j = 16 >> st;
        const uint32_t m = masks[st];
        const uint32_t p = __shfl_xor_sync(0xffffffffu, x, j);
        x = (lane & j) ? ((x & ~m) | ((p >> j) & m)) : ((x & m) | ((p & m) << j));
    }
    return x;
}

// Two own atoms (paired coordinates) against one candidate: r^2 - rlist^2
// for each, negative when the pair is listed.  The sign is exact: the chain
// ends in one rounding of a value that is zero only when r^2 = rlist^2.
__device__ __forceinline__ f2_t pair_r2m(f2_t jx2, f2_t jy2, f2_t jz2, float4 A, float2 Z, f2_t nrl2) {
    const f2_t ex = sub2(jx2, f2(A.x, A.y)), ey = sub2(jy2, f2(A.z, A.w)), ez = sub2(jz2, f2(Z.x, Z.y));
    return fma2(ez, ez, fma2(ey, ey, fma2(ex, ex, nrl2)));
}

// Hit bits of one candidate against the own atoms (bit i: own atom i).  One
// type: the own atoms in descending order, each sign bit shifted in from the
// bottom (one funnel shift per test).  Several types: the reference's t1 <=
// t2 loop (potential.rs:171-172) also decides, separately for each side --
// fwd: own atom i lists the candidate (type_j >= type_i); bwd: the candidate
// lists own atom i (type_i >= type_j).
template <bool SINGLE, bool BWD>
__device__ __forceinline__ void own_hits(f2_t jx2, f2_t jy2, f2_t jz2, int tj, int cpc4, const float4* own_xy,
                                         const float2* own_z, const int* own_t, f2_t nrl2, uint32_t& fwd,
                                         uint32_t& bwd) {
    fwd = 0u;
    bwd = 0u;
    if (SINGLE) {
        for (int i = cpc4 - 4; i >= 0; i -= 4) {
#pragma unroll
            for (int u = 2; u >= 0; u -= 2) {
                const f2_t h = pair_r2m(jx2, jy2, jz2, own_xy[(i + u) >> 1], own_z[(i + u) >> 1], nrl2);
                fwd = __funnelshift_l((unsigned)(h >> 32), fwd, 1);   // own atom i + u + 1
                fwd = __funnelshift_l((unsigned)h, fwd, 1);           // own atom i + u
            }
        }
        bwd = fwd;
    } else {
        for (int i = 0; i < cpc4; i += 4) {
            const uint32_t b0 = 1u << i;
#pragma unroll
            for (int u = 0; u < 4; u += 2) {
                const f2_t h = pair_r2m(jx2, jy2, jz2, own_xy[(i + u) >> 1], own_z[(i + u) >> 1], nrl2);
                const bool h0 = f2_lo(h) < 0.f, h1 = f2_hi(h) < 0.f;
                const int t0 = own_t[i + u], t1 = own_t[i + u + 1];
                if (h0 & (tj >= t0)) fwd |= b0 << u;
                if (h1 & (tj >= t1)) fwd |= b0 << (u + 1);
                if (BWD) {
                    if (h0 & (t0 >= tj)) bwd |= b0 << u;
                    if (h1 & (t1 >= tj)) bwd |= b0 << (u + 1);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The paired build's tests.  Shared memory per warp, in 32-bit words: the
// forward stream (A itself, then codes 14..26, at most 32 atoms a cell), the
// transposed hit rows [own atom][chunk], the own atoms (paired coordinates
// and types) and the 27 cell shifts.
constexpr int LM_WARPS = 4;
constexpr int LM_WIN = 14 * 32;
constexpr int LM_NQ = LM_WIN / 32;
constexpr int LM_MQ = LM_NQ + 1;     // odd: conflict-free columns
constexpr int LM_WARP_WORDS = LM_WIN + 32 * LM_MQ + 32 * 4 + 27 * 4 + 4;
static_assert((LM_WIN + 32 * LM_MQ) % 4 == 0 && LM_WARP_WORDS % 4 == 0, "float4 alignment");
constexpr int LM_CELL_MAX = 32;      // atoms a cell may hold for the paired build

template <bool SINGLE>
__global__ void __launch_bounds__(LM_WARPS * 32, 10) k_list_masks(Dev d) {
    if (*(volatile const unsigned int*)(d.bar + 2) == 0u) return;   // no rebuild this step
    if (chunk_failed(d) || d.direct_list) return;
    __shared__ __align__(16) uint32_t lm_smem[LM_WARPS * LM_WARP_WORDS];
    const unsigned FULL = 0xffffffffu;
    const int N = d.ntot;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t* cand = lm_smem + (size_t)wib * LM_WARP_WORDS;
    uint32_t* masks = cand + LM_WIN;
    float4* own_xy = reinterpret_cast<float4*>(masks + 32 * LM_MQ);
    float2* own_z = reinterpret_cast<float2*>(own_xy + 16);
    int* own_t = reinterpret_cast<int*>(own_z + 16);
    float4* tab = reinterpret_cast<float4*>(own_t + 32);
    const int gw = blockIdx.x * LM_WARPS + wib, nw = gridDim.x * LM_WARPS;
    // the cells of the rebuilding replicas the paired build takes (the step
    // kernel's work list, from position rb[1] on)
    const int m = d.rb[0], w0 = rb_cell_off(d)[d.rb[1]], nwork = rb_cell_off(d)[m];
    for (int wi = w0 + gw; wi < nwork; wi += nw) {
        const int i = rb_locate(rb_cell_off(d), m, wi);
        const int r = rb_rep(d)[i];
        const RepDev* W = d.rep + r;
        if (W->mode != MODE_CELLS) continue;
        const int c = W->cell_base + wi - rb_cell_off(d)[i];
        const float rl = (float)(W->rlist * (1.0 + 1e-5));
        const f2_t nrl2 = f2(-(rl * rl), -(rl * rl));
        const int nc[3] = {W->nc[0], W->nc[1], W->nc[2]};
        const int base = W->cell_base;
        const int local = c - base;
        if (local >= nc[0] * nc[1] * nc[2]) continue;   // a guard: the work list holds the grid only
        const long long rbeg = W->begin;
        const int rn = W->n;
        const int ib = d.cell_start[c], in = d.cell_count[c];
        if (ib < rbeg || ib + in > rbeg + rn) {
            if (lane == 0) atomicOr(d.err, E_CELLS);
            continue;
        }
        int ox, oy, oz;
        decode_cell(local, nc, ox, oy, oz);
        __syncwarp();
        // lane k < 27: neighbour cell with shift code k; its start, tagged
        // with the code, is what the expansion adds a bit position to
        int nb_start = 0, nb_cnt = 0;
        if (lane < 27) {
            const int dx = lane % 3 - 1, dy = (lane / 3) % 3 - 1, dz = lane / 9 - 1;
            int x = ox + dx; x = x < 0 ? x + nc[0] : (x >= nc[0] ? x - nc[0] : x);
            int y = oy + dy; y = y < 0 ? y + nc[1] : (y >= nc[1] ? y - nc[1] : y);
            int z = oz + dz; z = z < 0 ? z + nc[2] : (z >= nc[2] ? z - nc[2] : z);
            const int cj = base + (x * nc[1] + y) * nc[2] + z;
            nb_start = d.cell_start[cj];
            nb_cnt = d.cell_count[cj];
            if (nb_start < rbeg || nb_start + nb_cnt > rbeg + rn) {
                atomicOr(d.err, E_CELLS);
                nb_start = (int)rbeg;
                nb_cnt = 0;
            }
            d.nbs[(size_t)c * 27 + lane] = (uint32_t)nb_start | ((uint32_t)lane << IDX_BITS);
            tab[lane] = make_float4((float)dx * dbl_to_flt_rn(W->cs[0]), (float)dy * dbl_to_flt_rn(W->cs[1]),
                                    (float)dz * dbl_to_flt_rn(W->cs[2]), 0.f);
        }
        // a crowded cell anywhere in the rebuild: the direct build does it all
        if (__any_sync(FULL, nb_cnt > LM_CELL_MAX)) {
            if (lane == 0) atomicOr(d.bar + 4, 1u);
            continue;
        }
        // forward stream: A itself (code 13) first, then codes 14..26
        const int fcnt = lane >= CODE_ZERO && lane < 27 ? nb_cnt : 0;
        int incl = fcnt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, off);
            if (lane >= off) incl += v;
        }
        const int f_off = incl - fcnt;
        const int total = __shfl_sync(FULL, incl, 31);
        {
            const bool own = lane < in;
            const float4 xo = own ? d.mir[ib + lane] : make_float4(1e18f, 1e18f, 1e18f, __int_as_float(0x7fffffff));
            float* oxy = reinterpret_cast<float*>(own_xy) + ((lane >> 1) << 2) + (lane & 1);
            oxy[0] = xo.x;
            oxy[2] = xo.y;
            reinterpret_cast<float*>(own_z)[lane] = xo.z;
            own_t[lane] = type_of(xo);
        }
        if (fcnt > 0) {
            const uint32_t tag = (uint32_t)lane << IDX_BITS;
            for (int p = 0; p < fcnt; ++p) cand[f_off + p] = (uint32_t)(nb_start + p) | tag;
        }
        __syncwarp();
        const int nq = (total + 31) >> 5;
        const int cpc4 = (in + 3) & ~3;
        uint32_t e_n = 0u;
        float4 x_n = make_float4(0.f, 0.f, 0.f, 0.f);
        if (lane < total) {
            e_n = cand[lane];
            x_n = __ldg(d.mir + (e_n & IDX_MASK));
        }
        for (int q = 0; q < nq; ++q) {
            const bool valid = (q << 5) + lane < total;
            const uint32_t e = e_n;
            const float4 sh = tab[e >> IDX_BITS];
            const float jx = x_n.x + sh.x, jy = x_n.y + sh.y, jz = x_n.z + sh.z;
            const f2_t jx2 = f2(jx, jx), jy2 = f2(jy, jy), jz2 = f2(jz, jz);
            const int tj = type_of(x_n);
            if (((q + 1) << 5) + lane < total) {   // next chunk in flight
                e_n = cand[((q + 1) << 5) + lane];
                x_n = __ldg(d.mir + (e_n & IDX_MASK));
            }
            uint32_t fwd, bwd;
            own_hits<SINGLE, true>(jx2, jy2, jz2, tj, cpc4, own_xy, own_z, own_t, nrl2, fwd, bwd);
            if (!valid) fwd = bwd = 0u;
            // the forward cell's atom: its word for the opposite code
            const int code = (int)(e >> IDX_BITS);
            if (valid && code != CODE_ZERO) d.lmask[(size_t)(26 - code) * N + (e & IDX_MASK)] = bwd;
            masks[lane * LM_MQ + q] = warp_transpose32(fwd, lane);
        }
        __syncwarp();
        // A's words for codes 13..26: its row over the stream, cut at the
        // cells' offsets (a segment spans at most two chunks)
#pragma unroll 2
        for (int k = CODE_ZERO; k < 27; ++k) {
            const int off = __shfl_sync(FULL, f_off, k), cnt = __shfl_sync(FULL, nb_cnt, k);
            if (lane < in) {
                const uint32_t* row = masks + lane * LM_MQ;
                const int q0 = off >> 5, r0 = off & 31;
                uint32_t w = 0u;
                if (cnt > 0) {
                    w = row[q0] >> r0;
                    if (r0 != 0 && r0 + cnt > 32) w |= row[q0 + 1] << (32 - r0);
                    if (cnt < 32) w &= (1u << cnt) - 1u;
                }
                if (k == CODE_ZERO) w &= ~(1u << lane);   // the atom itself
                d.lmask[(size_t)k * N + ib + lane] = w;
            }
        }
    }
}

// The direct build: every cell against the stream of its 27 neighbour cells.
// all: every rebuilding replica (else those the paired build does not take).
template <bool SINGLE>
__device__ __forceinline__ void list_direct(const Dev& d, uint32_t* lb_smem, bool all) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t* cand = lb_smem + (size_t)wib * LB_WARP_WORDS;
    uint32_t* masks = cand + LB_WIN;
    // own atoms in pairs for the paired FP32 instructions: (x_2p, x_2p+1, y_2p,
    // y_2p+1), (z_2p, z_2p+1), and their types
    float4* own_xy = reinterpret_cast<float4*>(masks + 32 * LB_MQ);
    float2* own_z = reinterpret_cast<float2*>(own_xy + 16);
    int* own_t = reinterpret_cast<int*>(own_z + 16);
    float4* tab = reinterpret_cast<float4*>(own_t + 32);
    const int cap = d.cap;
    const int gw = blockIdx.x * LB_WARPS + wib, nw = gridDim.x * LB_WARPS;
    // the cells of the rebuilding replicas this build takes (the step
    // kernel's work list: all, or those before position rb[1])
    const int m = d.rb[0], nwork = rb_cell_off(d)[all ? m : d.rb[1]];
    for (int wi = gw; wi < nwork; wi += nw) {
        const int i = rb_locate(rb_cell_off(d), m, wi);
        const int r = rb_rep(d)[i];
        const RepDev* W = d.rep + r;
        if (W->mode != MODE_CELLS) continue;
        const int c = W->cell_base + wi - rb_cell_off(d)[i];
        const float rl = (float)(W->rlist * (1.0 + 1e-5));
        const f2_t nrl2 = f2(-(rl * rl), -(rl * rl));
        const int nc[3] = {W->nc[0], W->nc[1], W->nc[2]};
        const int base = W->cell_base;
        const int local = c - base;
        if (local >= nc[0] * nc[1] * nc[2]) continue;   // a guard: the work list holds the grid only
        const long long rbeg = W->begin;
        const int rn = W->n, tpa = W->tpa;
        const int ib = d.cell_start[c], in = d.cell_count[c];
        if (ib < rbeg || ib + in > rbeg + rn) {
            if (lane == 0) atomicOr(d.err, E_CELLS);
            continue;
        }
        if (in == 0) continue;
        int ox, oy, oz;
        decode_cell(local, nc, ox, oy, oz);
        __syncwarp();
        // lane k < 27: neighbour cell with shift code k
        int nb_start = 0, nb_cnt = 0;
        if (lane < 27) {
            const int dx = lane % 3 - 1, dy = (lane / 3) % 3 - 1, dz = lane / 9 - 1;
            int x = ox + dx; x = x < 0 ? x + nc[0] : (x >= nc[0] ? x - nc[0] : x);
            int y = oy + dy; y = y < 0 ? y + nc[1] : (y >= nc[1] ? y - nc[1] : y);
            int z = oz + dz; z = z < 0 ? z + nc[2] : (z >= nc[2] ? z - nc[2] : z);
            const int cj = base + (x * nc[1] + y) * nc[2] + z;
            nb_start = d.cell_start[cj];
            nb_cnt = d.cell_count[cj];
            if (nb_start < rbeg || nb_start + nb_cnt > rbeg + rn) {
                atomicOr(d.err, E_CELLS);
                nb_cnt = 0;
            }
            tab[lane] = make_float4((float)dx * dbl_to_flt_rn(W->cs[0]), (float)dy * dbl_to_flt_rn(W->cs[1]),
                                    (float)dz * dbl_to_flt_rn(W->cs[2]), 0.f);
        }
        int incl = nb_cnt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, off);
            if (lane >= off) incl += v;
        }
        const int nb_off = incl - nb_cnt;
        const int total = __shfl_sync(FULL, incl, 31);
        const int self_off = __shfl_sync(FULL, nb_off, CODE_ZERO);   // the own cell's segment
        int cmax = 0;
        for (int g = 0; g < in; g += 32) {
            const int cpc = min(32, in - g);
            const int s = ib + g + lane;
            const bool own = lane < cpc;
            __syncwarp();
            // rows past the cell's atoms (up to a multiple of 4) sit far away: no hits
            {
                const float4 xo = own ? d.mir[s] : make_float4(1e18f, 1e18f, 1e18f, __int_as_float(0x7fffffff));
                float* oxy = reinterpret_cast<float*>(own_xy) + ((lane >> 1) << 2) + (lane & 1);
                oxy[0] = xo.x;
                oxy[2] = xo.y;
                reinterpret_cast<float*>(own_z)[lane] = xo.z;
                own_t[lane] = type_of(xo);
            }
            const int cpc4 = (cpc + 3) & ~3;
            const int pself = self_off + g + lane;   // stream position of the atom itself
            int cnt = 0;
            // running output position: entry cnt of atom s is rowp[col],
            // rowp = segment + (cnt / tpa) * n * tpa + (s - begin) * tpa, col = cnt % tpa
            uint32_t* rowp = d.nbr + (size_t)cap * (size_t)rbeg + (size_t)(s - rbeg) * (size_t)tpa;
            const size_t rowstride = (size_t)rn * (size_t)tpa;
            int col = 0;
            for (int w0 = 0; w0 < total; w0 += LB_WIN) {
                const int wn = min(LB_WIN, total - w0);
                const int nq = (wn + 31) >> 5;
                __syncwarp();
                // lane k < 27 writes neighbour cell k's run of the window
                if (lane < 27) {
                    const int lo = max(nb_off, w0), hi = min(nb_off + nb_cnt, w0 + wn);
                    const uint32_t tag = (uint32_t)lane << IDX_BITS;
                    for (int p = lo; p < hi; ++p) cand[p - w0] = (uint32_t)(nb_start + p - nb_off) | tag;
                }
                __syncwarp();
                uint32_t e_n = 0u;
                float4 x_n = make_float4(0.f, 0.f, 0.f, 0.f);
                if (lane < wn) {
                    e_n = cand[lane];
                    x_n = __ldg(d.mir + (e_n & IDX_MASK));
                }
                for (int q = 0; q < nq; ++q) {
                    const bool valid = (q << 5) + lane < wn;
                    const float4 sh = tab[e_n >> IDX_BITS];
                    const float jx = x_n.x + sh.x, jy = x_n.y + sh.y, jz = x_n.z + sh.z;
                    const f2_t jx2 = f2(jx, jx), jy2 = f2(jy, jy), jz2 = f2(jz, jz);
                    const int tj = type_of(x_n);
                    if (((q + 1) << 5) + lane < wn) {   // next chunk in flight
                        e_n = cand[((q + 1) << 5) + lane];
                        x_n = __ldg(d.mir + (e_n & IDX_MASK));
                    }
                    // bit i of `mine`: own atom i lists this lane's candidate
                    uint32_t mine, unused;
                    own_hits<SINGLE, false>(jx2, jy2, jz2, tj, cpc4, own_xy, own_z, own_t, nrl2, mine, unused);
                    if (!valid) mine = 0u;
                    // 32x32 bit transpose across the warp: lane i gets bit k set when
                    // candidate k of the chunk hits own atom i
                    mine = warp_transpose32(mine, lane);
                    masks[lane * LB_MQ + q] = mine;
                }
                __syncwarp();
                // expansion: pass t appends entry t of every lane's atom, so the
                // stores of a pass land side by side
                uint32_t* myrow = masks + lane * LB_MQ;
                int tot = 0;
                if (own) {
                    const int ps = pself - w0;
                    if (ps >= 0 && ps < wn) myrow[ps >> 5] &= ~(1u << (ps & 31));
                    for (int q = 0; q < nq; ++q) tot += __popc(myrow[q]);
                }
                // entries this window writes (the rest of an overflowing list is
                // only counted)
                const int lim = max(0, min(tot, cap - cnt));
                int lmax = lim;
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) lmax = max(lmax, __shfl_xor_sync(FULL, lmax, off));
                if (tpa == 1) {
                    // masks bit-reversed: the next entry is the highest set bit
                    // (one find-leading-one), candidate 32 q + 31 - p
                    uint32_t mr = own ? __brev(myrow[0]) : 0u;
                    int qb = 31;
#pragma unroll 2
                    for (int t = 0; t < lmax; ++t) {
                        if (t < lim) {
                            while (mr == 0u) {   // t < lim <= tot: a set bit remains
                                qb += 32;
                                mr = __brev(myrow[qb >> 5]);
                            }
                            const int p = 31 - __clz(mr);
                            mr ^= 1u << p;
                            rowp[(size_t)t * rowstride] = cand[qb - p];
                        }
                    }
                    rowp += (size_t)tot * rowstride;
                } else {
                    uint32_t m = own ? myrow[0] : 0u;
                    int q = 0;
                    for (int t = 0; t < lmax; ++t) {
                        if (t < lim) {
                            while (m == 0u) m = myrow[++q];
                            const int k = __ffs(m) - 1;
                            m &= m - 1u;
                            rowp[col] = cand[(q << 5) + k];
                            if (++col == tpa) { col = 0; rowp += rowstride; }
                        }
                    }
                    // entries counted past the capacity are never written: no
                    // further window writes either (lim is 0 from here on)
                }
                cnt += tot;
            }
            if (own) {
                const int nfill = min(cnt, cap);
                if (d.refmode) sort_list_by_rank(d, s, nfill, tpa, rbeg, rn);
                d.nn[s] = nfill;
                if (cnt > cap) {
                    atomicOr(d.err, E_NLIST);
                    atomicMax(d.max_needed, cnt);
                }
            }
            cmax = max(cmax, cnt);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) cmax = max(cmax, __shfl_xor_sync(FULL, cmax, off));
        if (lane == 0 && cmax > 0) atomicMax(&d.rep[r].max_nn, cmax);
    }
}

// The paired build's expansion: lane = atom (32 consecutive atoms of one
// tile), the atom's 27 hit words and the tagged starts of its cell's 27
// neighbour cells staged in shared memory.
__device__ __forceinline__ void list_expand(const Dev& d, uint32_t* lb_smem) {
    const unsigned FULL = 0xffffffffu;
    const int N = d.ntot;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t* wm = lb_smem + (size_t)wib * LB_WARP_WORDS;   // [27][32] hit words
    uint32_t* wb = wm + 27 * 32;                              // [27][32] tagged neighbour-cell starts
    const int cap = d.cap;
    constexpr int GPT = TILE / 32;                            // warp groups per tile
    const int gw = blockIdx.x * LB_WARPS + wib, nw = gridDim.x * LB_WARPS;
    // the tiles of the rebuilding replicas the paired build takes (the step
    // kernel's work list, from position rb[1] on)
    const int m = d.rb[0], g0 = rb_tile_off(d)[d.rb[1]] * GPT, nwork = rb_tile_off(d)[m] * GPT;
    for (int g = g0 + gw; g < nwork; g += nw) {
        const int i = rb_locate(rb_tile_off(d), m, g / GPT);
        const int r = rb_rep(d)[i];
        const RepDev* W = d.rep + r;
        if (W->mode != MODE_CELLS) continue;
        const int4 tl = d.tiles[W->tile_begin + g / GPT - rb_tile_off(d)[i]];
        const int sub = (g % GPT) * 32;
        if (sub >= tl.z) continue;
        const long long rbeg = W->begin;
        const int rn = W->n, tpa = W->tpa;
        const int s = tl.y + sub + lane;
        bool own = sub + lane < tl.z;
        const int c = own ? d.cell[s] : 0;
        if (own && (c < W->cell_base || c >= W->cell_base + W->cell_cap)) {
            atomicOr(d.err, E_CELLS);
            own = false;
        }
        __syncwarp();
        // words kept bit-reversed (the next entry is then the leading one, a
        // single instruction); nz: the codes whose word has a hit, code k at
        // bit 31 - k
        int tot = 0;
        uint32_t nz = 0u;
#pragma unroll 9
        for (int k = 0; k < 27; ++k) {
            const uint32_t w = own ? __ldcs(d.lmask + (size_t)k * N + s) : 0u;
            wm[k * 32 + lane] = __brev(w);
            wb[k * 32 + lane] = own ? __ldg(d.nbs + (size_t)c * 27 + k) : 0u;
            tot += __popc(w);
            nz |= (w != 0u ? 0x80000000u : 0u) >> k;
        }
        __syncwarp();
        // entries written (the rest of an overflowing list is only counted)
        const int lim = min(tot, cap);
        int lmax = lim;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) lmax = max(lmax, __shfl_xor_sync(FULL, lmax, off));
        uint32_t* rowp = d.nbr + (size_t)cap * (size_t)rbeg + (size_t)(s - rbeg) * (size_t)tpa;
        const size_t rowstride = (size_t)rn * (size_t)tpa;
        // the next entry: lowest set bit of the current word; an exhausted
        // word moves on to the next code with a hit, in one step (t < lim <=
        // tot: a set bit remains)
        uint32_t m = 0u, b = 0u;
        if (tpa == 1) {
            uint32_t* wp = rowp;
#pragma unroll 2
            for (int t = 0; t < lmax; ++t) {
                if (t < lim) {
                    if (m == 0u) {
                        const int k = __clz(nz);
                        nz ^= 0x80000000u >> k;
                        m = wm[k * 32 + lane];
                        b = wb[k * 32 + lane];
                    }
                    const int p = __clz(m);
                    m ^= 0x80000000u >> p;
                    *wp = b + (uint32_t)p;
                }
                wp += rowstride;
            }
        } else {
            int col = 0;
            for (int t = 0; t < lmax; ++t) {
                if (t < lim) {
                    if (m == 0u) {
                        const int k = __clz(nz);
                        nz ^= 0x80000000u >> k;
                        m = wm[k * 32 + lane];
                        b = wb[k * 32 + lane];
                    }
                    const int p = __clz(m);
                    m ^= 0x80000000u >> p;
                    rowp[col] = b + (uint32_t)p;
                    if (++col == tpa) { col = 0; rowp += rowstride; }
                }
            }
        }
        if (own) {
            if (d.refmode) sort_list_by_rank(d, s, lim, tpa, rbeg, rn);
            d.nn[s] = lim;
            if (tot > cap) {
                atomicOr(d.err, E_NLIST);
                atomicMax(d.max_needed, tot);
            }
        }
        int cmax = own ? tot : 0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) cmax = max(cmax, __shfl_xor_sync(FULL, cmax, off));
        if (lane == 0 && cmax > 0) atomicMax(&d.rep[tl.x].max_nn, cmax);
    }
}

template <bool SINGLE>
// 11 blocks of 64 threads per SM (80 registers, shared memory for 11 blocks):
// latency-bound, so as many warps as fit (10 blocks / 95 registers: 0.7 %
// slower, for the direct build).
__global__ void __launch_bounds__(LB_WARPS * 32, 11) k_build_list(Dev d) {
    if (*(volatile const unsigned int*)(d.bar + 2) == 0u) return;   // no rebuild this step
    if (chunk_failed(d)) return;
    extern __shared__ __align__(16) uint32_t lb_smem[];
    __shared__ int s_last;
    // the paired build's masks are complete unless a cell was too crowded for them
    const bool direct = d.direct_list || *(volatile const unsigned int*)(d.bar + 4) != 0u;
    list_direct<SINGLE>(d, lb_smem, direct);
    if (!direct) list_expand(d, lb_smem);
    // The last block to finish closes the rebuild of every replica.
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(d.bar + 3, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (int r = threadIdx.x; r < d.nrep; r += blockDim.x) {
            RepDev* W = d.rep + r;
            if (W->rebuild) {
                W->rebuild = 0;
                W->nrebuilds += 1;
            }
        }
        if (threadIdx.x == 0) {
            if (d.trace) atomicAdd(d.trace + TR_LIST, global_ns() - d.trace[TR_STAMP]);
            if (direct) d.bar[5] += 1u;   // direct builds, for the engine's counters
            d.bar[4] = 0u;
            d.bar[3] = 0u;
            atomicExch(d.bar + 2, 0u);
        }
    }
}

// ---------------------------------------------------------------------------
// Host side.
constexpr int LB_SMEM = LB_WARPS * LB_WARP_WORDS * 4;

cudaError_t list_build_init() {
    cudaError_t err = cudaFuncSetAttribute(k_build_list<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, LB_SMEM);
    if (err != cudaSuccess) return err;
    return cudaFuncSetAttribute(k_build_list<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, LB_SMEM);
}

// Grid: every resident warp, no more than one per cell.
int list_build_grid(const Dev& d, int num_sms) {
    int bps = 0;
    const void* fn = d.single_type ? (const void*)k_build_list<true> : (const void*)k_build_list<false>;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, LB_WARPS * 32, LB_SMEM) != cudaSuccess) bps = 1;
    const int want = (d.ncells + LB_WARPS - 1) / LB_WARPS;
    return std::max(1, std::min(num_sms * std::max(bps, 1), want));
}

// The paired build's tests: every resident warp, no more than one per cell.
int list_masks_grid(const Dev& d, int num_sms) {
    int bps = 0;
    const void* fn = d.single_type ? (const void*)k_list_masks<true> : (const void*)k_list_masks<false>;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, LM_WARPS * 32, 0) != cudaSuccess) bps = 1;
    const int want = (d.ncells + LM_WARPS - 1) / LM_WARPS;
    return std::max(1, std::min(num_sms * std::max(bps, 1), want));
}

cudaError_t launch_list_build(const Dev& d, int grid, int mgrid, cudaStream_t st) {
    if (d.single_type) {
        k_list_masks<true><<<mgrid, LM_WARPS * 32, 0, st>>>(d);
        k_build_list<true><<<grid, LB_WARPS * 32, LB_SMEM, st>>>(d);
    } else {
        k_list_masks<false><<<mgrid, LM_WARPS * 32, 0, st>>>(d);
        k_build_list<false><<<grid, LB_WARPS * 32, LB_SMEM, st>>>(d);
    }
    return cudaGetLastError();
}

}  // namespace mdgb
