// host_util.cpp -- host-only helpers of libmdgb (no GPU needed).
//
//   mdgb_lj_new / mdgb_lj_eval   Potential::new_lennard_jones and
//                                get_potential_and_force (solver/src/solver/potential.rs:27-75)
//   mdgb_lattice                 U / FCC site order of initialize_particles_position
//                                (solver/src/initializer/position.rs:34-99)
//   mdgb_maxwell_boltzmann       initialize_velocities_maxwell_boltzmann
//                                (solver/src/initializer/velocity.rs:6-29), but seeded
//
// The reference draws velocities from an unseeded thread RNG; here the draw is
// seeded and bit-reproducible on every IEEE-754 host (x86_64 and aarch64):
// xoshiro256** (Blackman & Vigna 2018) seeded through splitmix64, normal
// deviates by the Marsaglia polar method, and a logarithm built from IEEE
// +,-,*,/ only (frexp reduction + atanh series), since libm's log is not
// guaranteed to round identically across platforms.  Compiled with
// -ffp-contract=off.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/mdgb.h"

namespace {

constexpr double K_B = 1.380648528;  // core/src/lib.rs:15

struct Xoshiro256 {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t& x) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    explicit Xoshiro256(uint64_t seed) {
        uint64_t x = seed;
        for (auto& v : s) v = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t result = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return result;
    }
    // uniform in [0, 1) with 53 random bits
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
};

// ln(x) for finite x > 0 from IEEE basic operations only.
double portable_log(double x) {
    int e = 0;
    double m = std::frexp(x, &e);  // x = m * 2^e, m in [0.5, 1), exact
    if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }  // m in [sqrt(1/2), sqrt(2))
    const double t = (m - 1.0) / (m + 1.0);
    const double t2 = t * t;
    // 2 atanh(t) = 2 (t + t^3/3 + t^5/5 + ...), |t| < 0.1716: 14 terms < 1e-22
    double sum = 0.0;
    for (int k = 27; k >= 1; k -= 2) sum = sum * t2 + 1.0 / (double)k;
    const double lm = 2.0 * t * sum;
    const double ln2_hi = 0.693147180369123816490;   // high bits of ln 2 (exact in 32 bits)
    const double ln2_lo = 1.90821492927058770002e-10;
    return ((double)e * ln2_hi + lm) + (double)e * ln2_lo;
}

// Marsaglia polar method: a pair of independent standard normal deviates.
void normal_pair(Xoshiro256& g, double& a, double& b) {
    for (;;) {
        const double u = 2.0 * g.uniform() - 1.0;
        const double v = 2.0 * g.uniform() - 1.0;
        const double s = u * u + v * v;
        if (s > 0.0 && s < 1.0) {
            const double f = std::sqrt(-2.0 * portable_log(s) / s);
            a = u * f;
            b = v * f;
            return;
        }
    }
}

void lj_eval(const double p[4], double r, double* u, double* dudr) {
    // potential.rs:57-75
    if (r > p[2]) { *u = 0.0; *dudr = 0.0; return; }
    const double s = p[0] / r;
    const double s2 = s * s;
    const double s4 = s2 * s2;
    const double s6 = s2 * s4;
    const double s12 = s6 * s6;
    *u = 4.0 * p[1] * (s12 - s6) - p[3];
    *dudr = (24.0 * p[1] / r) * (s6 - 2.0 * s12);
}

}  // namespace

extern "C" {

MDGB_API int mdgb_lj_new(double sigma, double eps, double out[4]) {
    if (!out || !(sigma > 0.0)) return MDGB_ERR_INVALID_ARGUMENT;
    double p[4] = {sigma, eps, sigma * 2.5, 0.0};  // potential.rs:28
    double u, f;
    lj_eval(p, p[2], &u, &f);                      // potential.rs:42
    out[0] = sigma; out[1] = eps; out[2] = p[2]; out[3] = u;
    return MDGB_OK;
}

MDGB_API int mdgb_lj_eval(const double pot[4], double r, double* u, double* dudr) {
    if (!pot || !u || !dudr) return MDGB_ERR_INVALID_ARGUMENT;
    lj_eval(pot, r, u, dudr);
    return MDGB_OK;
}

MDGB_API int mdgb_lattice(int kind, int64_t nx, int64_t ny, int64_t nz, double a, const double start[3],
                          double* out) {
    if (!out || nx < 0 || ny < 0 || nz < 0 || (kind != 0 && kind != 1)) return MDGB_ERR_INVALID_ARGUMENT;
    const double s0 = start ? start[0] : 0.0, s1 = start ? start[1] : 0.0, s2 = start ? start[2] : 0.0;
    for (int64_t x = 0; x < nx; ++x)
        for (int64_t y = 0; y < ny; ++y)
            for (int64_t z = 0; z < nz; ++z) {
                const int64_t cell = x * ny * nz + y * nz + z;   // position.rs:42-43
                const double X = (double)x, Y = (double)y, Z = (double)z;
                if (kind == 0) {
                    double* p = out + 3 * cell;
                    p[0] = s0 + X * a; p[1] = s1 + Y * a; p[2] = s2 + Z * a;
                } else {                                          // position.rs:60-96
                    double* p = out + 12 * cell;
                    p[0] = s0 + X * a;         p[1] = s1 + Y * a;         p[2] = s2 + Z * a;
                    p[3] = s0 + X * a;         p[4] = s1 + (Y + 0.5) * a; p[5] = s2 + (Z + 0.5) * a;
                    p[6] = s0 + (X + 0.5) * a; p[7] = s1 + Y * a;         p[8] = s2 + (Z + 0.5) * a;
                    p[9] = s0 + (X + 0.5) * a; p[10] = s1 + (Y + 0.5) * a; p[11] = s2 + Z * a;
                }
            }
    return MDGB_OK;
}

MDGB_API int mdgb_maxwell_boltzmann(int64_t n, double temperature, double mass, uint64_t seed,
                                    double* out_vel) {
    if (!out_vel || n < 0 || !(mass > 0.0) || temperature < 0.0) return MDGB_ERR_INVALID_ARGUMENT;
    // velocity.rs:8-10: T scaled to program units, sigma = sqrt(K_B T / m)
    const double t = temperature * 0.01;
    const double sigma = std::sqrt(K_B * t / mass);
    std::memset(out_vel, 0, sizeof(double) * 3 * (size_t)n);
    Xoshiro256 g(seed);
    const int64_t half = n / 2;
    double spare = 0.0;
    bool have = false;
    auto draw = [&]() {
        if (have) { have = false; return spare; }
        double a, b;
        normal_pair(g, a, b);
        spare = b; have = true;
        return a;
    };
    for (int64_t i = 0; i < half; ++i) {                  // velocity.rs:11-27
        const double x = sigma * draw(), y = sigma * draw(), z = sigma * draw();
        out_vel[3 * i] = x; out_vel[3 * i + 1] = y; out_vel[3 * i + 2] = z;
        out_vel[3 * (i + half)] = -x; out_vel[3 * (i + half) + 1] = -y; out_vel[3 * (i + half) + 2] = -z;
    }
    return MDGB_OK;
}

}  // extern "C"
