// Test helper: compares the engine's integer-op IEEE conversions
// (dbl_to_flt_rn, flt_to_dbl, fixed_to_double in mdgb_internal.cuh) with CUDA's conversion
// instructions, bit for bit, on random and edge-case inputs.  Prints the
// number of mismatches; exit status 0 when there are none.
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#include "../../moldyn_gb300/csrc/mdgb_internal.cuh"

using namespace mdgb;

__global__ void k_check(const double* in, int n, unsigned long long* bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = in[i];
    // fixed-point sum -> double: an int64 built from the input bits, scaled by 2^-27
    const long long q = (long long)(__double_as_longlong(x) >> (i % 13));
    const double f = fixed_to_double(q, 27);
    const double g = __ll2double_rn(q) * 0x1.0p-27;
    if (__double_as_longlong(f) != __double_as_longlong(g)) atomicAdd(bad + 2, 1ull);
    const float a = dbl_to_flt_rn(x);
    const float b = __double2float_rn(x);
    if (__float_as_uint(a) != __float_as_uint(b)) atomicAdd(bad, 1ull);
    const double c = flt_to_dbl(b);
    const double e = (double)b;
    if (__double_as_longlong(c) != __double_as_longlong(e)) atomicAdd(bad + 1, 1ull);
}

int main() {
    const int n = 1 << 22;
    double* h = new double[n];
    uint64_t s = 0x9E3779B97F4A7C15ull;
    for (int i = 0; i < n; ++i) {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        // magnitudes 2^-100 .. 2^100 with random mantissas, both signs
        const double m = 1.0 + (double)(s >> 12) * 0x1.0p-52;
        const int ex = (int)((s >> 3) % 201) - 100;
        double v = m * __builtin_ldexp(1.0, ex);
        if (s & 1) v = -v;
        // every 8th value is a float plus a half-ulp tie or near-tie
        if ((i & 7) == 0) {
            const float f = (float)v;
            const double ulp = __builtin_ldexp(1.0, __builtin_ilogb(f) - 23);
            v = (double)f + ((i & 8) ? 0.5 : 0.4999999) * ulp;
        }
        h[i] = v;
    }
    h[0] = 0.0; h[1] = -0.0; h[2] = 1.0; h[3] = -1.5; h[4] = 3.0e38; h[5] = 1.1754944e-38;
    double* d; unsigned long long* bad;
    cudaMalloc(&d, n * sizeof(double));
    cudaMalloc(&bad, 3 * sizeof(unsigned long long));
    cudaMemcpy(d, h, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemset(bad, 0, 3 * sizeof(unsigned long long));
    k_check<<<(n + 255) / 256, 256>>>(d, n, bad);
    unsigned long long hb[3] = {0, 0, 0};
    cudaError_t err = cudaMemcpy(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost);
    printf("dbl_to_flt mismatches %llu flt_to_dbl mismatches %llu fixed_to_double mismatches %llu status %s\n",
           hb[0], hb[1], hb[2], cudaGetErrorString(err));
    cudaFree(d); cudaFree(bad); delete[] h;
    return (err == cudaSuccess && hb[0] == 0 && hb[1] == 0 && hb[2] == 0) ? 0 : 1;
}
