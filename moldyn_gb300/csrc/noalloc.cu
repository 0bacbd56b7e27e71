// noalloc.cu -- mdgb_forces_noalloc: Lennard-Jones forces for callers that
// cannot allocate GPU memory.
//
// Who needs this: code that runs where cudaMalloc is not available to it --
// a plugin inside a host application that owns every device allocation
// through its own pool, a real-time loop where an allocation (which can
// synchronise the device) is not allowed, or a process whose memory budget
// is fixed up front.  Such a caller already holds its input and output
// buffers on the device and only needs the force evaluation itself.
//
// The entry point is a one-shot variant of the engine's force pass: it bins
// the atoms into a cell grid, orders each cell by atom index (a stable
// counting sort: every atom finds its rank among its cell's atoms in
// parallel), and evaluates the reference's FP64 Lennard-Jones arithmetic per
// pair over the neighbour cells.  Per-pair arithmetic is the reference's;
// the sums run cell by cell over the stencil rather than in the reference's
// ascending-j order, so results are deterministic and agree with the
// reference to about 1e-12 of the force scale, not bit for bit.  An axis
// shorter than three cut-off radii is one cell wide (no stencil along it);
// the other axes keep their cells.  Its scratch (cell counts, fill
// counters, cell starts, per-atom cell ids, the arrival order and the
// cell-sorted order) lives in one file-scope static __device__ array of
// fixed size, so the call allocates nothing.  That array exists on every GPU
// that loads the library and stays there until the process exits (about
// 1.2 MB).
//
// The host code never passes the array's name to a kernel (in host code it
// is only a stand-in, not a device address): once per device, with that
// device current, it asks the runtime for the array's device address with
// cudaGetSymbolAddress and passes that pointer.  The first call on a device
// does this set-up, so make the first call before any stream capture.
//
// All calls share the one array and every call leaves its contents behind;
// each call clears the counters it needs before use.  Calls that overlap on
// the GPU (on different streams, or from different threads) race on the
// array and give wrong results: serialise them.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/mdgb.h"

namespace {

constexpr int NA_MAX_ATOMS = MDGB_NOALLOC_MAX_ATOMS;
constexpr int NA_MAX_CELLS = MDGB_NOALLOC_MAX_CELLS;
constexpr int NA_MAX_SMALL_BOX = MDGB_NOALLOC_MAX_SMALL_BOX;
constexpr int NA_MAX_DEVICES = 64;
// layout (ints): counts[MAX_CELLS] fill[MAX_CELLS] starts[MAX_CELLS + 1]
//                cell_of[MAX_ATOMS] arrival[MAX_ATOMS] order[MAX_ATOMS]
constexpr size_t NA_WORDS = 3 * (size_t)NA_MAX_CELLS + 1 + 3 * (size_t)NA_MAX_ATOMS;

static __device__ __align__(256) int g_noalloc_scratch[NA_WORDS];

struct Scratch {
    int* counts;
    int* fill;
    int* starts;
    int* cell_of;
    int* arrival;   // atoms of each cell in atomic arrival order
    int* order;     // atoms of each cell in ascending index
};

__host__ __device__ inline Scratch carve(int* base) {
    Scratch s;
    s.counts = base;
    s.fill = base + NA_MAX_CELLS;
    s.starts = base + 2 * NA_MAX_CELLS;
    s.cell_of = base + 3 * NA_MAX_CELLS + 1;
    s.arrival = s.cell_of + NA_MAX_ATOMS;
    s.order = s.arrival + NA_MAX_ATOMS;
    return s;
}

struct Grid {
    int nc[3];
    double box[3];
    double inv_cs[3];
};

std::mutex g_mu;
int* g_scratch_ptr[NA_MAX_DEVICES] = {};

__global__ void k_na_clear(Scratch s, int ncells) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncells) { s.counts[c] = 0; s.fill[c] = 0; }
}

// Cell of a position.  Positions are expected in [0, box); a coordinate
// outside is taken to its periodic image, and a non-finite one lands in cell
// 0 of that axis, so the index is always inside the grid.
__device__ __forceinline__ int cell_index(const double* p, const Grid& g) {
    int c[3];
    for (int a = 0; a < 3; ++a) {
        const double q = floor(p[a] * g.inv_cs[a]);
        const double n = (double)g.nc[a];
        double w = q - n * floor(q / n);        // periodic image of the cell coordinate
        if (!(w >= 0.0)) w = 0.0;               // NaN / inf
        if (w > n - 1.0) w = n - 1.0;
        c[a] = (int)w;
    }
    return (c[0] * g.nc[1] + c[1]) * g.nc[2] + c[2];
}

__global__ void k_na_bin(const double* pos, int n, Grid g, Scratch s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cell_index(pos + 3 * (size_t)i, g);
    s.cell_of[i] = c;
    atomicAdd(s.counts + c, 1);
}

// exclusive scan of the cell counts by one block
__global__ void k_na_scan(Scratch s, int ncells) {
    __shared__ int part[1024];
    const int per = (ncells + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per, b1 = min(b0 + per, ncells);
    int sum = 0;
    for (int c = b0; c < b1; ++c) sum += s.counts[c];
    part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int k = 0; k < (int)blockDim.x; ++k) { const int t = part[k]; part[k] = run; run += t; }
        s.starts[ncells] = run;
    }
    __syncthreads();
    int run = part[threadIdx.x];
    for (int c = b0; c < b1; ++c) { s.starts[c] = run; run += s.counts[c]; }
}

__global__ void k_na_scatter(int n, Scratch s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = s.cell_of[i];
    s.arrival[s.starts[c] + atomicAdd(s.fill + c, 1)] = i;
}

// Stable order inside each cell: atom i's slot is the number of atoms of its
// cell with a smaller index, found by every atom in parallel from the
// arrival list (no serial per-cell sort), so the sums run in a fixed order.
__global__ void k_na_rank(int n, Scratch s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = s.cell_of[i];
    const int b = s.starts[c], m = s.counts[c];
    int rank = 0;
    for (int k = 0; k < m; ++k) rank += s.arrival[b + k] < i;
    s.order[b + rank] = i;
}

// update_force (solver/src/solver/potential.rs:158-216) for one particle type:
// the reference's single-shift minimum image, |r| <= r_cut, and its FP64
// operation sequence for U and dU/dr.  An axis of one cell has no stencil.
__global__ void k_na_force(const double* pos, int n, Grid g, Scratch s, double sigma, double eps4,
                           double eps24, double rc, double ucut, double* force, double* potential,
                           double* temp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double px = pos[3 * (size_t)i], py = pos[3 * (size_t)i + 1], pz = pos[3 * (size_t)i + 2];
    const int ci = s.cell_of[i];
    const int cz = ci % g.nc[2], cy = (ci / g.nc[2]) % g.nc[1], cx = ci / (g.nc[1] * g.nc[2]);
    const int rx0 = g.nc[0] == 1 ? 0 : -1, ry0 = g.nc[1] == 1 ? 0 : -1, rz0 = g.nc[2] == 1 ? 0 : -1;
    double fx = 0.0, fy = 0.0, fz = 0.0, pe = 0.0, vr = 0.0;
    const double hx = 0.5 * g.box[0], hy = 0.5 * g.box[1], hz = 0.5 * g.box[2];
    for (int dz = rz0; dz <= -rz0; ++dz)
        for (int dy = ry0; dy <= -ry0; ++dy)
            for (int dx = rx0; dx <= -rx0; ++dx) {
                const int x = (cx + dx + g.nc[0]) % g.nc[0], y = (cy + dy + g.nc[1]) % g.nc[1],
                          z = (cz + dz + g.nc[2]) % g.nc[2];
                const int c = (x * g.nc[1] + y) * g.nc[2] + z;
                const int b = s.starts[c], e = b + s.counts[c];
                for (int k = b; k < e; ++k) {
                    const int j = s.order[k];
                    if (j == i) continue;
                    double rx = __dsub_rn(pos[3 * (size_t)j], px);
                    double ry = __dsub_rn(pos[3 * (size_t)j + 1], py);
                    double rz = __dsub_rn(pos[3 * (size_t)j + 2], pz);
                    if (rx < -hx) rx = __dadd_rn(rx, g.box[0]); else if (rx > hx) rx = __dsub_rn(rx, g.box[0]);
                    if (ry < -hy) ry = __dadd_rn(ry, g.box[1]); else if (ry > hy) ry = __dsub_rn(ry, g.box[1]);
                    if (rz < -hz) rz = __dadd_rn(rz, g.box[2]); else if (rz > hz) rz = __dsub_rn(rz, g.box[2]);
                    const double r = __dsqrt_rn(
                        __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz)));
                    if (r > rc) continue;
                    const double sr = __ddiv_rn(sigma, r);
                    const double s2 = __dmul_rn(sr, sr);
                    const double s4 = __dmul_rn(s2, s2);
                    const double s6 = __dmul_rn(s2, s4);
                    const double s12 = __dmul_rn(s6, s6);
                    const double u = __dsub_rn(__dmul_rn(eps4, __dsub_rn(s12, s6)), ucut);
                    const double dudr = __dmul_rn(__ddiv_rn(eps24, r), __dsub_rn(s6, __dmul_rn(2.0, s12)));
                    const double gx = __dmul_rn(__ddiv_rn(rx, r), dudr);
                    const double gy = __dmul_rn(__ddiv_rn(ry, r), dudr);
                    const double gz = __dmul_rn(__ddiv_rn(rz, r), dudr);
                    fx = __dadd_rn(fx, gx); fy = __dadd_rn(fy, gy); fz = __dadd_rn(fz, gz);
                    pe = __dadd_rn(pe, u);
                    vr = __dadd_rn(vr, __dadd_rn(__dadd_rn(__dmul_rn(gx, rx), __dmul_rn(gy, ry)), __dmul_rn(gz, rz)));
                }
            }
    force[3 * (size_t)i] = fx; force[3 * (size_t)i + 1] = fy; force[3 * (size_t)i + 2] = fz;
    if (potential) potential[i] = pe;
    if (temp) temp[i] = vr;
}

}  // namespace

// Cells per axis: at least r_cut wide; an axis shorter than three cells is
// one cell (no stencil along it); the others are coarsened together until the
// grid fits MDGB_NOALLOC_MAX_CELLS.  Host only.  Returns false for a box or
// cut-off that is not positive and finite.
static bool noalloc_grid(const double box[3], double r_cut, int nc_out[3]) {
    if (!(r_cut > 0.0) || !std::isfinite(r_cut)) return false;
    for (int a = 0; a < 3; ++a)
        if (!(box[a] > 0.0) || !std::isfinite(box[a])) return false;
    long long nc[3];
    for (int a = 0; a < 3; ++a) {
        double q = std::floor(box[a] / (r_cut * (1.0 + 1e-9)));
        if (!(q >= 0.0)) q = 0.0;
        if (q > (double)NA_MAX_CELLS) q = (double)NA_MAX_CELLS;   // clamp before the cast
        nc[a] = (long long)q;
        if (nc[a] < 3) nc[a] = 1;
    }
    // coarsen: every multi-cell axis by the same factor, then (where the
    // three-cell floor kept the grid too large) the largest axis takes the
    // whole remaining factor at once -- a few rounds at most
    const long long prod0 = nc[0] * nc[1] * nc[2];
    if (prod0 > NA_MAX_CELLS) {
        int k = 0;
        for (int a = 0; a < 3; ++a) k += nc[a] >= 3;
        const double f = std::pow((double)NA_MAX_CELLS / (double)prod0, 1.0 / k);
        for (int a = 0; a < 3; ++a)
            if (nc[a] >= 3) {
                const long long m = (long long)std::floor((double)nc[a] * f);
                nc[a] = m < 3 ? 3 : m;
            }
    }
    for (int round = 0; round < 8 && nc[0] * nc[1] * nc[2] > NA_MAX_CELLS; ++round) {
        int a = 0;
        if (nc[1] > nc[a]) a = 1;
        if (nc[2] > nc[a]) a = 2;
        const long long rest = nc[0] * nc[1] * nc[2] / nc[a];
        long long want = NA_MAX_CELLS / rest;
        if (want < 3) want = 3;
        nc[a] = want < nc[a] ? want : nc[a];
    }
    if (nc[0] * nc[1] * nc[2] > NA_MAX_CELLS) return false;   // unreachable: 27 cells fit
    for (int a = 0; a < 3; ++a) nc_out[a] = (int)nc[a];
    return true;
}

extern "C" MDGB_API int mdgb_forces_noalloc(int64_t n, const double* d_pos, const double box[3], double sigma,
                                            double eps, double* d_force, double* d_potential, double* d_temp,
                                            void* stream) {
    if (n < 0 || (n > 0 && (!d_pos || !d_force)) || !box || !(sigma > 0.0) || !std::isfinite(sigma) ||
        !std::isfinite(eps))
        return MDGB_ERR_INVALID_ARGUMENT;
    for (int a = 0; a < 3; ++a)
        if (!(box[a] > 0.0) || !std::isfinite(box[a])) return MDGB_ERR_INVALID_ARGUMENT;
    if (n > NA_MAX_ATOMS) return MDGB_ERR_NOALLOC_TOO_LARGE;
    if (n == 0) return MDGB_OK;
    // Potential::new_lennard_jones (potential.rs:27-55), on the host
    double lj[4];
    mdgb_lj_new(sigma, eps, lj);
    const double rc = lj[2], ucut = lj[3];
    Grid g;
    int nc[3];
    if (!noalloc_grid(box, rc, nc)) return MDGB_ERR_INVALID_ARGUMENT;
    for (int a = 0; a < 3; ++a) {
        g.nc[a] = nc[a];
        g.box[a] = box[a];
        g.inv_cs[a] = (double)nc[a] / box[a];
    }
    const int ncells = g.nc[0] * g.nc[1] * g.nc[2];
    // a box under three cut-off radii on every axis is one cell: every pair is
    // tested, so the atom count is bounded (a liquid that small holds a few
    // hundred atoms)
    if (ncells == 1 && n > NA_MAX_SMALL_BOX) return MDGB_ERR_NOALLOC_TOO_LARGE;

    // once per device, with that device current: the scratch array's device address
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return MDGB_ERR_CUDA;
    int* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return MDGB_ERR_CUDA;
            g_scratch_ptr[dev] = static_cast<int*>(p);
        }
        base = g_scratch_ptr[dev];
    }
    Scratch s = carve(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int N = (int)n;
    const int tb = 256;
    const double eps4 = 4.0 * eps, eps24 = 24.0 * eps;
    // each launch's own status (cudaLaunchKernel returns it), so an error the
    // host application left pending is neither reported nor cleared here
    void* a_clear[] = {&s, (void*)&ncells};
    void* a_bin[] = {(void*)&d_pos, &N, &g, &s};
    void* a_scan[] = {&s, (void*)&ncells};
    void* a_scat[] = {&N, &s};
    void* a_force[] = {(void*)&d_pos, &N, &g, &s, &sigma, (void*)&eps4, (void*)&eps24, (void*)&rc, (void*)&ucut,
                       &d_force, &d_potential, &d_temp};
    const unsigned gc = (unsigned)((ncells + tb - 1) / tb), ga = (unsigned)((N + tb - 1) / tb);
    cudaError_t ce = cudaLaunchKernel((const void*)k_na_clear, dim3(gc), dim3(tb), a_clear, 0, st);
    if (ce == cudaSuccess) ce = cudaLaunchKernel((const void*)k_na_bin, dim3(ga), dim3(tb), a_bin, 0, st);
    if (ce == cudaSuccess) ce = cudaLaunchKernel((const void*)k_na_scan, dim3(1), dim3(1024), a_scan, 0, st);
    if (ce == cudaSuccess) ce = cudaLaunchKernel((const void*)k_na_scatter, dim3(ga), dim3(tb), a_scat, 0, st);
    if (ce == cudaSuccess) ce = cudaLaunchKernel((const void*)k_na_rank, dim3(ga), dim3(tb), a_scat, 0, st);
    if (ce == cudaSuccess)
        ce = cudaLaunchKernel((const void*)k_na_force, dim3((unsigned)((N + 127) / 128)), dim3(128), a_force, 0, st);
    return ce == cudaSuccess ? MDGB_OK : MDGB_ERR_CUDA;
}
