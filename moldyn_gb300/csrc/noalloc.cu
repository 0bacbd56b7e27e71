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
// the atoms into a cell grid, orders each cell, and evaluates the reference's
// FP64 Lennard-Jones arithmetic over the 27 neighbour cells.  Its scratch
// (cell counts, cell starts, per-atom cell ids, the cell-sorted atom order)
// lives in one file-scope static __device__ array of fixed size, so the call
// allocates nothing.  That array exists on every GPU that loads the library
// and stays there until the process exits (about 0.9 MB).
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
constexpr int NA_MAX_DEVICES = 64;
// layout (ints): counts[MAX_CELLS] fill[MAX_CELLS] starts[MAX_CELLS + 1]
//                cell_of[MAX_ATOMS] order[MAX_ATOMS]
constexpr size_t NA_WORDS = 3 * (size_t)NA_MAX_CELLS + 1 + 2 * (size_t)NA_MAX_ATOMS;

static __device__ __align__(256) int g_noalloc_scratch[NA_WORDS];

struct Scratch {
    int* counts;
    int* fill;
    int* starts;
    int* cell_of;
    int* order;
};

__host__ __device__ inline Scratch carve(int* base) {
    Scratch s;
    s.counts = base;
    s.fill = base + NA_MAX_CELLS;
    s.starts = base + 2 * NA_MAX_CELLS;
    s.cell_of = base + 3 * NA_MAX_CELLS + 1;
    s.order = s.cell_of + NA_MAX_ATOMS;
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

__device__ __forceinline__ int cell_index(const double* p, const Grid& g) {
    int c[3];
    for (int a = 0; a < 3; ++a) {
        int k = (int)floor(p[a] * g.inv_cs[a]);
        k %= g.nc[a];
        if (k < 0) k += g.nc[a];
        c[a] = k;
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
    s.order[s.starts[c] + atomicAdd(s.fill + c, 1)] = i;
}

// ascending atom index inside each cell, so the sums run in a fixed order
__global__ void k_na_sort(Scratch s, int ncells) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    int* o = s.order + s.starts[c];
    const int m = s.counts[c];
    for (int a = 1; a < m; ++a) {
        const int e = o[a];
        int k = a - 1;
        while (k >= 0 && o[k] > e) { o[k + 1] = o[k]; --k; }
        o[k + 1] = e;
    }
}

// update_force (solver/src/solver/potential.rs:158-216) for one particle type:
// the reference's single-shift minimum image, |r| <= r_cut, and its FP64
// operation sequence for U and dU/dr.
__global__ void k_na_force(const double* pos, int n, Grid g, Scratch s, double sigma, double eps4,
                           double eps24, double rc, double ucut, double* force, double* potential,
                           double* temp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double px = pos[3 * (size_t)i], py = pos[3 * (size_t)i + 1], pz = pos[3 * (size_t)i + 2];
    const int ci = s.cell_of[i];
    const int cz = ci % g.nc[2], cy = (ci / g.nc[2]) % g.nc[1], cx = ci / (g.nc[1] * g.nc[2]);
    const bool single = g.nc[0] == 1;
    const int lo = single ? 0 : -1, hi = single ? 0 : 1;
    double fx = 0.0, fy = 0.0, fz = 0.0, pe = 0.0, vr = 0.0;
    const double hx = 0.5 * g.box[0], hy = 0.5 * g.box[1], hz = 0.5 * g.box[2];
    for (int dz = lo; dz <= hi; ++dz)
        for (int dy = lo; dy <= hi; ++dy)
            for (int dx = lo; dx <= hi; ++dx) {
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

extern "C" MDGB_API int mdgb_forces_noalloc(int64_t n, const double* d_pos, const double box[3], double sigma,
                                            double eps, double* d_force, double* d_potential, double* d_temp,
                                            void* stream) {
    if (n < 0 || (n > 0 && (!d_pos || !d_force)) || !box || !(sigma > 0.0)) return MDGB_ERR_INVALID_ARGUMENT;
    for (int a = 0; a < 3; ++a)
        if (!(box[a] > 0.0)) return MDGB_ERR_INVALID_ARGUMENT;
    if (n > NA_MAX_ATOMS) return MDGB_ERR_NOALLOC_TOO_LARGE;
    if (n == 0) return MDGB_OK;
    // Potential::new_lennard_jones (potential.rs:27-55), on the host
    double lj[4];
    mdgb_lj_new(sigma, eps, lj);
    const double rc = lj[2], ucut = lj[3];
    // cell grid: cells at least r_cut wide; a box under three cells per axis uses one cell
    Grid g;
    long long nc[3];
    bool single = false;
    for (int a = 0; a < 3; ++a) {
        nc[a] = (long long)std::floor(box[a] / (rc * (1.0 + 1e-9)));
        if (nc[a] < 3) single = true;
    }
    if (!single)
        while (nc[0] * nc[1] * nc[2] > NA_MAX_CELLS) {
            int a = 0;
            if (nc[1] > nc[a]) a = 1;
            if (nc[2] > nc[a]) a = 2;
            --nc[a];
        }
    if (single || nc[0] < 3 || nc[1] < 3 || nc[2] < 3) nc[0] = nc[1] = nc[2] = 1;
    for (int a = 0; a < 3; ++a) {
        g.nc[a] = (int)nc[a];
        g.box[a] = box[a];
        g.inv_cs[a] = (double)nc[a] / box[a];
    }
    const int ncells = g.nc[0] * g.nc[1] * g.nc[2];

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
    const Scratch s = carve(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int N = (int)n;
    const int tb = 256;
    k_na_clear<<<(ncells + tb - 1) / tb, tb, 0, st>>>(s, ncells);
    k_na_bin<<<(N + tb - 1) / tb, tb, 0, st>>>(d_pos, N, g, s);
    k_na_scan<<<1, 1024, 0, st>>>(s, ncells);
    k_na_scatter<<<(N + tb - 1) / tb, tb, 0, st>>>(N, s);
    k_na_sort<<<(ncells + tb - 1) / tb, tb, 0, st>>>(s, ncells);
    k_na_force<<<(N + 127) / 128, 128, 0, st>>>(d_pos, N, g, s, sigma, 4.0 * eps, 24.0 * eps, rc, ucut, d_force,
                                                d_potential, d_temp);
    return cudaGetLastError() == cudaSuccess ? MDGB_OK : MDGB_ERR_CUDA;
}
