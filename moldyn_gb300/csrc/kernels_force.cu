// kernels_force.cu -- Lennard-Jones pair forces over the Verlet list.
//
// Replaces update_force (solver/src/solver/potential.rs:158-216): per atom i
// the force F_i = sum_j r_ij/|r_ij| * dU/dr(|r_ij|), the potential sum
// U_i = sum_j U(|r_ij|) and temp_i = sum_j F_ij . r_ij over every j with
// |r_ij| <= r_cut, r_ij = x_j - x_i taken to the image picked by the
// reference's single-shift rule (potential.rs:186-200).
//
// k_force_fp64  -- the plain path.  Every pair is evaluated with the
//   reference's FP64 operation sequence through explicit round-to-nearest
//   intrinsics (no contraction), so each pair term carries the reference's
//   bits; with MDGB_FLAG_REFERENCE_ORDER the list is in the reference's j
//   order and the per-atom sums are bit-identical too.  An FP32 prefilter on
//   the mirror skips candidates that are certainly outside r_cut.
// k_force_mixed -- the chosen path.  FP32 pair maths from the float4 mirror
//   (cell-relative coordinates, periodic cell shift from the list entry),
//   force sums in deterministic 64-bit fixed point, potential/virial in FP32
//   per atom (FP64 across atoms).  An atom with a pair whose FP32 r^2 lies
//   within 1e-5 of r_cut^2 is left whole to k_force_band, which decides those
//   pairs with the reference's FP64 arithmetic, so the set of interacting
//   pairs equals the reference's.
//
// Both end with the second half kick v += F dt/2m (integrator.rs:49-55) when
// called from a step, and on NVE chunks with the next step's first kick and
// drift (kick_and_drift).  TPA threads share one atom's list; their partial
// sums are combined by a fixed shuffle tree.  The fused passes of an NVE chunk
// (NOE) neither sum the per-atom potential and virial nor store them or the
// forces (both kicks take the forces from registers): the chunk's last,
// unfused pass writes all three, and nothing reads them in between.  The
// kick/drift FP64 helpers get the FMA-or-not choice as a compile-time
// constant (a run-time flag made the compiler issue both forms).
#include "mdgb_internal.cuh"

namespace mdgb {

__device__ __forceinline__ void shift_table(float4* tab, const RepDev* R) {
    if (threadIdx.x < 27) {
        const int c = threadIdx.x;
        const float dx = (float)(c % 3 - 1), dy = (float)((c / 3) % 3 - 1), dz = (float)(c / 9 - 1);
        tab[c] = make_float4(dx * (float)R->cs[0], dy * (float)R->cs[1], dz * (float)R->cs[2], 0.f);
    }
}

// The reference's FP64 displacement and distance (potential.rs:181-201).
__device__ __forceinline__ double ref_distance(const double4_32a pi, const double4_32a pj, const double* box,
                                               double& rx, double& ry, double& rz) {
    rx = __dsub_rn(pj.x, pi.x);
    ry = __dsub_rn(pj.y, pi.y);
    rz = __dsub_rn(pj.z, pi.z);
    const double hx = 0.5 * box[0], hy = 0.5 * box[1], hz = 0.5 * box[2];
    if (rx < -hx) rx = __dadd_rn(rx, box[0]); else if (rx > hx) rx = __dsub_rn(rx, box[0]);
    if (ry < -hy) ry = __dadd_rn(ry, box[1]); else if (ry > hy) ry = __dsub_rn(ry, box[1]);
    if (rz < -hz) rz = __dadd_rn(rz, box[2]); else if (rz > hz) rz = __dsub_rn(rz, box[2]);
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
    return __dsqrt_rn(r2);
}

// ---------------------------------------------------------------------------
// 64-bit fixed-point accumulation without float->int64 conversions (those run
// on GB300's narrow FP64 pipe).  A term v (float, already scaled to fixed-point
// units) is split exactly as v = h * 2^23 + l with h = rint(v / 2^23) and
// l = v - h * 2^23 (|l| <= 2^22, exact in FP32).  Both are rounded to integers
// by the magic-number method: adding M = 1.5 * 2^23 to a float of magnitude
// <= 2^22 lands in [2^23, 2^24], where the float's bit pattern is
// bits(M) + rint(x).  Each term's bit pattern minus bits(M) is summed modulo
// 2^32 (one three-input add per word), so
//     sum_k rint(v_k) = (sum h_k) * 2^23 + sum l_k
// exactly, in any order, for |v| <= 2^44 (the kernel re-accumulates an atom
// with exact conversions when one of its terms may be larger).
constexpr float FIX_MAGIC = 12582912.0f;           // 1.5 * 2^23
constexpr unsigned FIX_MAGIC_BITS = 0x4B400000u;   // bits of FIX_MAGIC
constexpr int FIX_FOLD = 256;                      // most terms per lane the words can hold

struct FixAcc {
    unsigned hi, lo;
    __device__ __forceinline__ void init() { hi = lo = 0u; }
    // With at most FIX_FOLD terms the two 32-bit words cannot overflow
    // (|h| <= 2^21, |l| <= 2^22 per term).
    __device__ __forceinline__ long long total() const {
        return ((long long)(int)hi << 23) + (long long)(int)lo;
    }
};

// One term per accumulator pair, with the term already divided by 2^23
// (t = v / 2^23; the scaling is exact): a = t + M holds M + rint(t) = M + h,
// l' = t - h is exact (Sterbenz) and fma(l', 2^23, M) = M + rint(v - h 2^23).
// The x and y components go through the paired instructions together.
__device__ __forceinline__ void fix_add_xyz(FixAcc& ax, FixAcc& ay, FixAcc& az, f2_t dxy, float dz, float g) {
    const f2_t M2 = f2(FIX_MAGIC, FIX_MAGIC);
    const f2_t K2 = f2(8388608.0f, 8388608.0f);
    const f2_t t2 = mul2(dxy, f2(g, g));
    const f2_t a2 = add2(t2, M2);
    const f2_t l2 = sub2(t2, sub2(a2, M2));
    const f2_t b2 = fma2(l2, K2, M2);
    ax.hi += (unsigned)a2 - FIX_MAGIC_BITS;
    ay.hi += (unsigned)(a2 >> 32) - FIX_MAGIC_BITS;
    ax.lo += (unsigned)b2 - FIX_MAGIC_BITS;
    ay.lo += (unsigned)(b2 >> 32) - FIX_MAGIC_BITS;
    const float tz = dz * g;
    const float az_ = tz + FIX_MAGIC;
    const float lz = tz - (az_ - FIX_MAGIC);
    const float bz = fmaf(lz, 8388608.0f, FIX_MAGIC);
    az.hi += __float_as_uint(az_) - FIX_MAGIC_BITS;
    az.lo += __float_as_uint(bz) - FIX_MAGIC_BITS;
}

template <int TPA>
__device__ __forceinline__ long long tpa_sum_ll(long long v) {
#pragma unroll
    for (int off = TPA / 2; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off, TPA);
    return v;
}
template <int TPA>
__device__ __forceinline__ double tpa_sum_d(double v) {
#pragma unroll
    for (int off = TPA / 2; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off, TPA);
    return v;
}
template <int TPA>
__device__ __forceinline__ float tpa_sum_f(float v) {
#pragma unroll
    for (int off = TPA / 2; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off, TPA);
    return v;
}

// The next tile of this launch's tile list: one per block, or (persistent)
// from a work counter over the list, costliest tiles first.
__device__ __forceinline__ int next_tile(const Dev& d, bool persistent, int& iter, int* s_tile) {
    if (!persistent) return (iter++ == 0 && (int)blockIdx.x < d.ntile_list) ? d.tile_list[blockIdx.x] : -1;
    __syncthreads();
    if (threadIdx.x == 0) *s_tile = (int)atomicAdd(d.queue + d.list_class, 1u);
    __syncthreads();
    const int q = *s_tile;
    if (q >= d.ntile_list) return -1;
    return d.tile_list[q];
}

// Second half kick v += F dt/2m (integrator.rs:49-55).  With sp.fused (NVE
// chunks) also the next step's first half kick and drift (integrator.rs:30-46)
// into the other position/mirror buffers -- the step kernel that follows only
// decides and rebuilds.  Same operations, in the same order, as the unfused
// kick and drift.  Returns the displacement since the last rebuild.
// FM: the mixed path's fused multiply-adds (a compile-time constant).
template <bool FM>
__device__ __forceinline__ float kick_and_drift(const Dev& d, const StepParams& sp, const RepDev* R,
                                                const float* tcs, int s, int ty, double fx, double fy,
                                                double fz) {
    const int N = d.ntot;
    constexpr bool fm = FM;
    const double c = sp.kick_c[ty];
    double vx = madd(d.vel[s], fx, c, fm);
    double vy = madd(d.vel[N + s], fy, c, fm);
    double vz = madd(d.vel[2 * N + s], fz, c, fm);
    float disp = 0.f;
    if (sp.fused) {
        vx = madd(vx, fx, c, fm);
        vy = madd(vy, fy, c, fm);
        vz = madd(vz, fz, c, fm);
        const double4_32a p = drift_wrap(d.pos[s], vx, vy, vz, sp.dt, R->box, fm);
        d.pos_next[s] = p;
        const int cl = d.cell[s] - R->cell_base;
        if (cl >= 0 && cl < R->nc[0] * R->nc[1] * R->nc[2]) {
            const float4 m = mirror_of(p, cl, *R, tcs + 3, fm);
            d.mir_next[s] = m;
            disp = mirror_disp(m, d.mir0[s], tcs);
        } else {
            atomicOr(d.err, E_CELLS);
        }
    }
    d.vel[s] = vx;
    d.vel[N + s] = vy;
    d.vel[2 * N + s] = vz;
    return disp;
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Largest displacement of the warp into the replica's running maximum.
__device__ __forceinline__ void note_displacement(const Dev& d, int r, float disp) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) disp = fmaxf(disp, __shfl_xor_sync(0xffffffffu, disp, off));
    if ((threadIdx.x & 31) == 0 && disp > 0.f) atomicMax(&d.rep[r].max_disp_bits, __float_as_uint(disp));
}

// ---------------------------------------------------------------------------
template <int TPA, bool KICK, bool PERSIST>
__global__ void __launch_bounds__(TILE * TPA) k_force_fp64(Dev d, StepParams sp) {
    if (chunk_failed(d)) return;
    __shared__ float4 tab[27];
    __shared__ float tcs[8];
    __shared__ int s_tile;
    const int N = d.ntot;
    const int a = threadIdx.x / TPA, lane = threadIdx.x % TPA;
    int iter = 0;
    for (;;) {
        const int t = next_tile(d, PERSIST, iter, &s_tile);
        if (t < 0) break;
        const int4 tl = d.tiles[t];
        const RepDev* R = d.rep + tl.x;
        const long long rbeg = R->begin;
        const int rn = R->n;
        __syncthreads();
        shift_table(tab, R);
        if (KICK && sp.fused && threadIdx.x == 0) drift_consts(*R, tcs);
        __syncthreads();
        const double box[3] = {R->box[0], R->box[1], R->box[2]};
        const float Lf[3] = {(float)box[0], (float)box[1], (float)box[2]};
        const bool brute = R->mode == MODE_BRUTE;
        const int s = tl.y + a;
        const bool act = a < tl.z;
        double fx = 0.0, fy = 0.0, fz = 0.0, pe = 0.0, vr = 0.0;
        int ty = 0;
        if (act) {
            const double4_32a pi = d.pos[s];
            const float4 mi = d.mir[s];
            ty = type_of(pi);
            const int n = d.nn[s];
            for (int k = lane; k < n; k += TPA) {
                const uint32_t e = __ldcs(d.nbr + list_index(s, k, TPA, rbeg, rn, d.cap));
                const int j = (int)(e & IDX_MASK);
                const PairDev& P = d.pair[ty * MAX_TYPES + type_of(__ldg(d.mir + j))];
                // FP32 prefilter (certainly outside r_cut -> skip)
                {
                    const float4 mj = __ldg(d.mir + j);
                    const float4 sh = tab[e >> IDX_BITS];
                    float ex = mj.x - mi.x + sh.x, ey = mj.y - mi.y + sh.y, ez = mj.z - mi.z + sh.z;
                    if (brute) {
                        if (ex < -0.5f * Lf[0]) ex += Lf[0]; else if (ex > 0.5f * Lf[0]) ex -= Lf[0];
                        if (ey < -0.5f * Lf[1]) ey += Lf[1]; else if (ey > 0.5f * Lf[1]) ey -= Lf[1];
                        if (ez < -0.5f * Lf[2]) ez += Lf[2]; else if (ez > 0.5f * Lf[2]) ez -= Lf[2];
                    }
                    if (ex * ex + ey * ey + ez * ez > P.rc2f_hi * 1.0001f) continue;
                }
                const double4_32a pj = d.pos[j];
                double rx, ry, rz;
                const double r = ref_distance(pi, pj, box, rx, ry, rz);
                if (r > P.rc) continue;                                          // :202-204
                // potential.rs:57-75 get_potential_and_force
                const double sr = __ddiv_rn(P.sigma, r);
                const double s2 = __dmul_rn(sr, sr);
                const double s4 = __dmul_rn(s2, s2);
                const double s6 = __dmul_rn(s2, s4);
                const double s12 = __dmul_rn(s6, s6);
                const double u = __dsub_rn(__dmul_rn(P.eps4, __dsub_rn(s12, s6)), P.ucut);
                const double dudr = __dmul_rn(__ddiv_rn(P.eps24, r), __dsub_rn(s6, __dmul_rn(2.0, s12)));
                // :207-211
                const double gx = __dmul_rn(__ddiv_rn(rx, r), dudr);
                const double gy = __dmul_rn(__ddiv_rn(ry, r), dudr);
                const double gz = __dmul_rn(__ddiv_rn(rz, r), dudr);
                const double tt = __dadd_rn(__dadd_rn(__dmul_rn(gx, rx), __dmul_rn(gy, ry)), __dmul_rn(gz, rz));
                fx = __dadd_rn(fx, gx); fy = __dadd_rn(fy, gy); fz = __dadd_rn(fz, gz);
                pe = __dadd_rn(pe, u);
                vr = __dadd_rn(vr, tt);
            }
        }
        if (TPA > 1) {
            fx = tpa_sum_d<TPA>(fx); fy = tpa_sum_d<TPA>(fy); fz = tpa_sum_d<TPA>(fz);
            pe = tpa_sum_d<TPA>(pe); vr = tpa_sum_d<TPA>(vr);
        }
        float disp = 0.f;
        if (act && lane == 0) {
            d.frc[s] = fx; d.frc[N + s] = fy; d.frc[2 * N + s] = fz;
            d.epot[s] = pe; d.evir[s] = vr;
            if (KICK) disp = kick_and_drift<false>(d, sp, R, tcs, s, ty, fx, fy, fz);   // integrator.rs:49-55
        }
        if (KICK && sp.fused) note_displacement(d, tl.x, disp);
    }
}

// ---------------------------------------------------------------------------
// Mixed path.  The per-pair FP32 maths is shared by the loops below.
struct PairF {
    float sig2, eps4, eps24, ucut, rc2_lo, rc2_hi;
};

__device__ __forceinline__ PairF pairf(const PairDev& P) {
    return PairF{P.sig2f, P.eps4f, P.eps24f, P.ucutf, P.rc2f_lo, P.rc2f_hi};
}

// LJ for one pair at displacement (dx,dy,dz): fs = (dU/dr)/r, u = U(r).
__device__ __forceinline__ void lj_f32(const PairF& P, float r2, float& fs, float& u) {
    const float r2i = __fdividef(1.0f, r2);
    const float s2 = P.sig2 * r2i;
    const float s6 = s2 * s2 * s2;
    // (24 eps / r^2) s6 (1 - 2 s6) = (dU/dr) / r ;  4 eps s6 (s6 - 1) - u_cut = U
    fs = P.eps24 * r2i * s6 * fmaf(-2.0f, s6, 1.0f);
    u = fmaf(P.eps4 * s6, s6 - 1.0f, -P.ucut);
}

// NAIVE: the FP32-naive variant of the precision study -- force sums in plain
// FP32 registers instead of fixed point (same pair maths).
template <bool NAIVE, bool NOE = false>
struct MixedAcc {
    FixAcc ax, ay, az;
    float fx, fy, fz;
    float pe, vr, gmax;
    __device__ __forceinline__ void init() {
        ax.init(); ay.init(); az.init();
        fx = fy = fz = 0.f;
        pe = vr = gmax = 0.f;
    }
    // fscale_t: the fixed-point scale divided by 2^23; gmax tracks |fs| * fscale_t
    __device__ __forceinline__ void add(f2_t dxy, float dz, float r2, float fs, float u, float fscale_t) {
        if (!NOE) {
            pe += u;
            vr = fmaf(fs, r2, vr);
        }
        if (NAIVE) {
            fx = fmaf(f2_lo(dxy), fs, fx); fy = fmaf(f2_hi(dxy), fs, fy); fz = fmaf(dz, fs, fz);
            return;
        }
        const float g = fs * fscale_t;
        gmax = fmaxf(gmax, fabsf(g));
        fix_add_xyz(ax, ay, az, dxy, dz, g);
    }
    __device__ __forceinline__ void add(float dx, float dy, float dz, float r2, float fs, float u, float fscale_t) {
        add(f2(dx, dy), dz, r2, fs, u, fscale_t);
    }
};

// The reference's minimum image of one FP64 displacement component
// (potential.rs:186-200: r < -L/2 -> r + L, r > L/2 -> r - L) with the
// comparisons on the bit patterns (L/2 exact: exponent - 1): integer work
// instead of GB300's narrow FP64 pipe.
__device__ __forceinline__ double min_image_ref(double r, double L) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(r);
    const unsigned long long mag = b & 0x7FFFFFFFFFFFFFFFull;
    const unsigned long long half = (unsigned long long)__double_as_longlong(L) - (1ull << 52);
    if (mag > half) return dadd_nospec(r, (b >> 63) ? L : -L);
    return r;
}

// The reference's FP64 decision for one pair (potential.rs:181-204: the
// minimum-image displacement, r = sqrt(r^2), interacting when r <= r_cut);
// on success (dx,dy,dz) is the FP64 displacement rounded to FP32.  No square
// root: sqrt_rn(r^2) <= r_cut exactly when r^2 < rc2_cut, the smallest double
// whose correctly rounded square root exceeds r_cut (computed on the host).
__device__ __forceinline__ bool exact_pair(const Dev& d, const RepDev* R, int s, int j, const PairDev& PD,
                                           float& dx, float& dy, float& dz) {
    const double4_32a pi = d.pos[s], pj = d.pos[j];
    const double rx = min_image_ref(__dsub_rn(pj.x, pi.x), R->box[0]);
    const double ry = min_image_ref(__dsub_rn(pj.y, pi.y), R->box[1]);
    const double rz = min_image_ref(__dsub_rn(pj.z, pi.z), R->box[2]);
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
    // both non-negative: the bit patterns order like the values
    if (__double_as_longlong(r2) >= __double_as_longlong(PD.rc2_cut)) return false;
    dx = dbl_to_flt_rn(rx); dy = dbl_to_flt_rn(ry); dz = dbl_to_flt_rn(rz);
    return true;
}

template <int TPA, bool SINGLE, bool KICK, bool PERSIST, bool NAIVE = false, bool NOE = false>
// 9 blocks of 128 threads per SM (56 registers): the kernel is latency-bound
// on its neighbour gathers, so it keeps as many warps resident as it can.  The
// variants that also sum potential and virial need two more registers than
// that allows (at 56 they spill): 8 blocks, 64 registers.
__global__ void __launch_bounds__(TILE * TPA, ((NOE ? 9 : 8) / TPA) > 0 ? ((NOE ? 9 : 8) / TPA) : 1)
    k_force_mixed(Dev d, StepParams sp) {
    if (chunk_failed(d)) return;
    __shared__ float4 tab[27];
    __shared__ float tcs[8];
    __shared__ int s_tile;
    const int N = d.ntot;
    const int a = threadIdx.x / TPA, lane = threadIdx.x % TPA;
    const float fscale = d.fscale;
    const float fscale_t = NAIVE ? 1.0f : fscale * 1.1920928955078125e-07f;   // fscale / 2^23 (exact)
    // each term |dx * g| <= rlist * gmax; the magic-number split is exact up to
    // 2^44 fixed-point units, i.e. |t| <= 2^21 after the division by 2^23
    const float rl = (float)(d.rlist * 1.01);
    const float split_limit = 2097152.0f / rl;       // 2^44 / 2^23 / rlist
    const float range_limit = 4294967296.0f / rl;    // 2^55 / 2^23 / rlist
    int iter = 0;
    for (;;) {
        const int t = next_tile(d, PERSIST, iter, &s_tile);
        if (t < 0) break;
        const int4 tl = d.tiles[t];
        const RepDev* R = d.rep + tl.x;
        const long long rbeg = R->begin;
        const int rn = R->n;
        __syncthreads();
        shift_table(tab, R);
        if (KICK && sp.fused && threadIdx.x == 0) drift_consts(*R, tcs);
        __syncthreads();
        const bool brute = R->mode == MODE_BRUTE;
        const int s = tl.y + a;
        const bool act = a < tl.z;
        if (KICK && act && lane == 0) {
            // the epilogue's operands: in L2 by the time the pair loop is done
            prefetch_l2(d.vel + s);
            prefetch_l2(d.vel + N + s);
            prefetch_l2(d.vel + 2 * N + s);
            if (sp.fused) {
                prefetch_l2(d.pos + s);
                prefetch_l2(d.mir0 + s);
                prefetch_l2(d.cell + s);
            }
        }
        MixedAcc<NAIVE, NOE> acc;
        acc.init();
        int ty = 0, n_own = 0;
        bool deferred = false;   // an atom with a pair in the band goes to k_force_band whole
        if (act) {
            const float4 xi = d.mir[s];
            ty = type_of(xi);
            PairF P0{};
            if (SINGLE) P0 = pairf(d.pair[ty * MAX_TYPES + ty]);
            const int n = d.nn[s];
            n_own = n;
            if (!brute) {
                // hot loop: FP32 and integer work only, two candidates in flight
                bool band = false;
                const f2_t xixy = f2(xi.x, xi.y);
                auto pair = [&](uint32_t e, float4 xj) {
                    const float4 sh = tab[e >> IDX_BITS];
                    const f2_t dxy = add2(sub2(f2(xj.x, xj.y), xixy), f2(sh.x, sh.y));
                    const float dz = xj.z - xi.z + sh.z;
                    const PairF P = SINGLE ? P0 : pairf(d.pair[ty * MAX_TYPES + type_of(xj)]);
                    const float dx = f2_lo(dxy), dy = f2_hi(dxy);
                    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                    if (r2 >= P.rc2_lo) {
                        // within 1e-5 of r_cut^2: the atom is finished by k_force_band
                        band |= r2 <= P.rc2_hi;
                        return;
                    }
                    float fs, u;
                    lj_f32(P, r2, fs, u);
                    acc.add(dxy, dz, r2, fs, u, fscale_t);
                };
                // this lane's entries k = lane, lane + TPA, ...: two per iteration,
                // the next iteration's two list words already in flight (the list
                // streams from HBM; the gathers hit L2)
                const uint32_t* lbase = d.nbr + list_index(s, lane, TPA, rbeg, rn, d.cap);
                const size_t lstride = (size_t)rn * TPA;
                const int m = n > lane ? (n - lane + TPA - 1) / TPA : 0;
                uint32_t ea = 0u, eb = 0u;
                if (m > 0) ea = __ldcs(lbase);
                if (m > 1) eb = __ldcs(lbase + lstride);
                int i = 0;
                for (; i + 1 < m; i += 2) {
                    const float4 xa = __ldg(d.mir + (ea & IDX_MASK));
                    const float4 xb = __ldg(d.mir + (eb & IDX_MASK));
                    uint32_t na = 0u, nb = 0u;
                    if (i + 2 < m) na = __ldcs(lbase + (size_t)(i + 2) * lstride);
                    if (i + 3 < m) nb = __ldcs(lbase + (size_t)(i + 3) * lstride);
                    pair(ea, xa);
                    pair(eb, xb);
                    ea = na;
                    eb = nb;
                }
                if (i < m) pair(ea, __ldg(d.mir + (ea & IDX_MASK)));
                deferred = band;
            } else {
                // brute mode (a box smaller than three list radii): the reference's
                // FP64 displacement for every pair -- these replicas are tiny
                for (int k = lane; k < n; k += TPA) {
                    const uint32_t e = __ldcs(d.nbr + list_index(s, k, TPA, rbeg, rn, d.cap));
                    const int j = (int)(e & IDX_MASK);
                    const PairDev& PD = d.pair[ty * MAX_TYPES + type_of(__ldg(d.mir + j))];
                    float dx, dy, dz;
                    if (!exact_pair(d, R, s, j, PD, dx, dy, dz)) continue;
                    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                    float fs, u;
                    lj_f32(pairf(PD), r2, fs, u);
                    acc.add(dx, dy, dz, r2, fs, u, fscale_t);
                }
            }
        }
        if (TPA > 1) {
#pragma unroll
            for (int off = TPA / 2; off > 0; off >>= 1) deferred |= __shfl_xor_sync(0xffffffffu, deferred, off, TPA);
        }
        if (deferred && lane == 0) {
            const int slot = atomicAdd(d.band_count, 1);
            d.band_list[slot] = make_int2(s, tl.x);
        }
        long long sx = acc.ax.total(), sy = acc.ay.total(), sz = acc.az.total();
        // terms this lane summed: at most its share of the list
        const int nl = act && n_own > lane ? (n_own - lane + TPA - 1) / TPA : 0;
        if (!NAIVE && act && !deferred && (acc.gmax > split_limit || nl > FIX_FOLD)) {
            // a term may exceed the exact range of the split, or the lane summed
            // more terms than the 32-bit words hold: redo this lane's terms with
            // exact float -> int64 conversions (very close pairs, huge lists)
            if (acc.gmax > range_limit) atomicOr(d.err, E_FIXED);
            sx = sy = sz = 0;
            const float4 xi = d.mir[s];
            const int n = d.nn[s];
            for (int k = lane; k < n; k += TPA) {
                const uint32_t e = __ldcs(d.nbr + list_index(s, k, TPA, rbeg, rn, d.cap));
                const int j = (int)(e & IDX_MASK);
                const float4 xj = __ldg(d.mir + j);
                const float4 sh = tab[e >> IDX_BITS];
                float dx = xj.x - xi.x + sh.x, dy = xj.y - xi.y + sh.y, dz = xj.z - xi.z + sh.z;
                const PairDev& PD = d.pair[ty * MAX_TYPES + type_of(xj)];
                const PairF P = pairf(PD);
                if (brute) {
                    if (!exact_pair(d, R, s, j, PD, dx, dy, dz)) continue;
                } else {
                    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                    if (r2 > P.rc2_hi) continue;
                    if (r2 >= P.rc2_lo && !exact_pair(d, R, s, j, PD, dx, dy, dz)) continue;
                }
                const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                float fs, u;
                lj_f32(P, r2, fs, u);
                const float g = fs * fscale;
                sx += __float2ll_rn(dx * g);
                sy += __float2ll_rn(dy * g);
                sz += __float2ll_rn(dz * g);
            }
        }
        float pe = acc.pe, vr = acc.vr;
        float nfx = acc.fx, nfy = acc.fy, nfz = acc.fz;
        if (TPA > 1) {
            if (NAIVE) {
                nfx = tpa_sum_f<TPA>(nfx); nfy = tpa_sum_f<TPA>(nfy); nfz = tpa_sum_f<TPA>(nfz);
            } else {
                sx = tpa_sum_ll<TPA>(sx); sy = tpa_sum_ll<TPA>(sy); sz = tpa_sum_ll<TPA>(sz);
            }
            if (!NOE) { pe = tpa_sum_f<TPA>(pe); vr = tpa_sum_f<TPA>(vr); }
        }
        float disp = 0.f;
        if (act && lane == 0 && !deferred) {
            const double fx = NAIVE ? flt_to_dbl(nfx) : fixed_to_double(sx, d.fscale_log2);
            const double fy = NAIVE ? flt_to_dbl(nfy) : fixed_to_double(sy, d.fscale_log2);
            const double fz = NAIVE ? flt_to_dbl(nfz) : fixed_to_double(sz, d.fscale_log2);
            if (!NOE) {
                d.frc[s] = fx; d.frc[N + s] = fy; d.frc[2 * N + s] = fz;
                d.epot[s] = flt_to_dbl(pe); d.evir[s] = flt_to_dbl(vr);
            }
            if (KICK) disp = kick_and_drift<true>(d, sp, R, tcs, s, ty, fx, fy, fz);
        }
        if (KICK && sp.fused) note_displacement(d, tl.x, disp);
    }
}

// ---------------------------------------------------------------------------
// Atoms with a pair whose FP32 r^2 lies within 1e-5 of r_cut^2 (about one in
// six hundred per step): k_force_mixed leaves them (and their kick/drift) to
// this kernel, so its hot loop carries no FP64 code and no second pass
// (an inline second pass cost ~9 % of the force kernel's time although it
// almost never ran).  One warp per atom, lanes over the list; the band pairs
// are decided with the reference's FP64 arithmetic (no square root: the
// r^2 threshold of exact_pair); every term is rounded to fixed point exactly as in
// k_force_mixed (rint(dx * g), here by the conversion instruction), so the
// force sums are the ones the main kernel would have produced.  Potential and
// temp are FP32 sums in a fixed shuffle order.
template <bool NAIVE>
__global__ void __launch_bounds__(128) k_force_band(Dev d, StepParams sp, int kick) {
    if (chunk_failed(d)) return;
    const int N = d.ntot;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int count = *(volatile const int*)d.band_count;
    const float fscale = d.fscale;
    const float rl = (float)(d.rlist * 1.01);
    const float range_limit = 36028797018963968.0f / rl;   // 2^55 / rlist
    for (int w = gw; w < count; w += nw) {
        const int2 sr = d.band_list[w];
        const int s = sr.x;
        const RepDev* R = d.rep + sr.y;
        const long long rbeg = R->begin;
        const int rn = R->n, tpa = R->tpa;
        const float csf[3] = {(float)R->cs[0], (float)R->cs[1], (float)R->cs[2]};
        const float4 xi = d.mir[s];
        const int ty = type_of(xi);
        const int n = d.nn[s];
        if (kick && lane == 0) {   // the epilogue's operands, on their way
            prefetch_l2(d.vel + s);
            prefetch_l2(d.vel + N + s);
            prefetch_l2(d.vel + 2 * N + s);
            if (sp.fused) {
                prefetch_l2(d.pos + s);
                prefetch_l2(d.mir0 + s);
                prefetch_l2(d.cell + s);
            }
        }
        long long sx = 0, sy = 0, sz = 0;
        float fx = 0.f, fy = 0.f, fz = 0.f, pe = 0.f, vr = 0.f;
        bool over = false;
        // this lane's list words and neighbour mirrors, all loads issued before
        // the maths (the warp handles one atom: latency is the whole cost)
        constexpr int KB = 4;
        uint32_t eb[KB];
        float4 xb[KB];
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            const int k = lane + 32 * q;
            eb[q] = k < n ? __ldcs(d.nbr + list_index(s, k, tpa, rbeg, rn, d.cap)) : 0u;
        }
#pragma unroll
        for (int q = 0; q < KB; ++q) xb[q] = __ldg(d.mir + (eb[q] & IDX_MASK));
        auto entry = [&](uint32_t e, float4 xj) {
            const int j = (int)(e & IDX_MASK);
            const int c = (int)(e >> IDX_BITS);
            // the shift table of the main kernel (shift_table)
            const float shx = (float)(c % 3 - 1) * csf[0], shy = (float)((c / 3) % 3 - 1) * csf[1],
                        shz = (float)(c / 9 - 1) * csf[2];
            const f2_t dxy = add2(sub2(f2(xj.x, xj.y), f2(xi.x, xi.y)), f2(shx, shy));
            float dx = f2_lo(dxy), dy = f2_hi(dxy), dz = xj.z - xi.z + shz;
            const PairDev& PD = d.pair[ty * MAX_TYPES + type_of(xj)];
            const PairF P = pairf(PD);
            const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            if (r2 > P.rc2_hi) return;
            float rr2 = r2;
            if (r2 >= P.rc2_lo) {
                if (!exact_pair(d, R, s, j, PD, dx, dy, dz)) return;
                rr2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            }
            float fs, u;
            lj_f32(P, rr2, fs, u);
            pe += u;
            vr = fmaf(fs, rr2, vr);
            if (NAIVE) {
                fx = fmaf(dx, fs, fx); fy = fmaf(dy, fs, fy); fz = fmaf(dz, fs, fz);
            } else {
                const float g = fs * fscale;
                over |= fabsf(g) > range_limit;
                sx += __float2ll_rn(dx * g);
                sy += __float2ll_rn(dy * g);
                sz += __float2ll_rn(dz * g);
            }
        };
#pragma unroll
        for (int q = 0; q < KB; ++q)
            if (lane + 32 * q < n) entry(eb[q], xb[q]);
        for (int k = lane + 32 * KB; k < n; k += 32) {
            const uint32_t e = __ldcs(d.nbr + list_index(s, k, tpa, rbeg, rn, d.cap));
            entry(e, __ldg(d.mir + (e & IDX_MASK)));
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            sx += __shfl_down_sync(0xffffffffu, sx, off);
            sy += __shfl_down_sync(0xffffffffu, sy, off);
            sz += __shfl_down_sync(0xffffffffu, sz, off);
            fx += __shfl_down_sync(0xffffffffu, fx, off);
            fy += __shfl_down_sync(0xffffffffu, fy, off);
            fz += __shfl_down_sync(0xffffffffu, fz, off);
            pe += __shfl_down_sync(0xffffffffu, pe, off);
            vr += __shfl_down_sync(0xffffffffu, vr, off);
        }
        if (over) atomicOr(d.err, E_FIXED);
        if (lane == 0) {
            const double Fx = NAIVE ? flt_to_dbl(fx) : fixed_to_double(sx, d.fscale_log2);
            const double Fy = NAIVE ? flt_to_dbl(fy) : fixed_to_double(sy, d.fscale_log2);
            const double Fz = NAIVE ? flt_to_dbl(fz) : fixed_to_double(sz, d.fscale_log2);
            d.frc[s] = Fx; d.frc[N + s] = Fy; d.frc[2 * N + s] = Fz;
            d.epot[s] = flt_to_dbl(pe); d.evir[s] = flt_to_dbl(vr);
            if (kick) {
                float tcs[8];
                drift_consts(*R, tcs);
                const float disp = kick_and_drift<true>(d, sp, R, tcs, s, ty, Fx, Fy, Fz);
                if (sp.fused && disp > 0.f) atomicMax(&d.rep[sr.y].max_disp_bits, __float_as_uint(disp));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host-side launch table.  precision: 0 FP64 plain, 1 mixed, 2 FP32-naive.
using force_fn = void (*)(Dev, StepParams);

template <int TPA, bool KICK, bool PERSIST>
static force_fn pick_mixed(bool single, bool naive, bool noe) {
    if constexpr (KICK) {
        if (noe && !naive)
            return single ? (force_fn)k_force_mixed<TPA, true, true, PERSIST, false, true>
                          : (force_fn)k_force_mixed<TPA, false, true, PERSIST, false, true>;
    }
    if (naive)
        return single ? (force_fn)k_force_mixed<TPA, true, KICK, PERSIST, true>
                      : (force_fn)k_force_mixed<TPA, false, KICK, PERSIST, true>;
    return single ? (force_fn)k_force_mixed<TPA, true, KICK, PERSIST>
                  : (force_fn)k_force_mixed<TPA, false, KICK, PERSIST>;
}

template <int TPA, bool PERSIST>
static force_fn pick_tpa(int precision, bool single, bool kick, bool noe) {
    if (precision != 0) {
        const bool naive = precision == 2;
        return kick ? pick_mixed<TPA, true, PERSIST>(single, naive, noe)
                    : pick_mixed<TPA, false, PERSIST>(single, naive, noe);
    }
    return kick ? (force_fn)k_force_fp64<TPA, true, PERSIST> : (force_fn)k_force_fp64<TPA, false, PERSIST>;
}

template <bool PERSIST>
static force_fn pick_persist(int tpa, int precision, bool single, bool kick, bool noe) {
    switch (tpa) {
        case 1: return pick_tpa<1, PERSIST>(precision, single, kick, noe);
        case 2: return pick_tpa<2, PERSIST>(precision, single, kick, noe);
        case 4: return pick_tpa<4, PERSIST>(precision, single, kick, noe);
        case 8: return pick_tpa<8, PERSIST>(precision, single, kick, noe);
        default: return nullptr;
    }
}

using band_fn = void (*)(Dev, StepParams, int);
band_fn band_kernel(int precision) {
    if (precision == 0) return nullptr;
    return precision == 2 ? (band_fn)k_force_band<true> : (band_fn)k_force_band<false>;
}

// noe: a fused NVE pass (no per-atom potential/virial); mixed path only.
force_fn force_kernel(int tpa, int precision, bool single, bool kick, bool persistent, bool noe) {
    return persistent ? pick_persist<true>(tpa, precision, single, kick, noe)
                      : pick_persist<false>(tpa, precision, single, kick, noe);
}

}  // namespace mdgb
