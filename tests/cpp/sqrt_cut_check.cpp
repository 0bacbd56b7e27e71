// Test helper: the r^2 threshold of the mixed path's exact pair test
// (sqrt_cut in moldyn_gb300/csrc/host_math.h) against its definition.  For
// each cutoff rc: sqrt(t) > rc, sqrt(t^-) <= rc for the double t^- below t,
// and (sqrt(r2) <= rc) == (r2 < t) for every r2 within 2000 ulps of t.
// Prints the number of failures; exit status 0 when there are none.
#include <cmath>
#include <cstdint>
#include <cstdio>

#include "../../moldyn_gb300/csrc/host_math.h"

int main() {
    long bad = 0, checked = 0;
    uint64_t s = 0x2545F4914F6CDD1Dull;
    double cuts[4000];
    int n = 0;
    const double fixed[] = {2.5, 0.85, 0.3405 * 2.5, 0.3418 * 2.5, 1.0, 2.0, 1.122462048309373, 3.0, 1e-3, 1e3};
    for (double c : fixed) cuts[n++] = c;
    while (n < 4000) {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        cuts[n++] = std::ldexp(1.0 + (double)(s >> 12) * 0x1.0p-52, (int)((s >> 2) % 21) - 10);
    }
    for (int i = 0; i < n; ++i) {
        const double rc = cuts[i];
        const double t = mdgb::sqrt_cut(rc);
        if (!(std::sqrt(t) > rc) || !(std::sqrt(std::nextafter(t, 0.0)) <= rc)) ++bad;
        double r2 = t;
        for (int k = 0; k < 2000; ++k) r2 = std::nextafter(r2, 0.0);
        for (int k = 0; k < 4000; ++k, r2 = std::nextafter(r2, INFINITY)) {
            ++checked;
            if ((std::sqrt(r2) <= rc) != (r2 < t)) ++bad;
        }
    }
    std::printf("sqrt_cut: %ld failures in %ld checks\n", bad, checked);
    return bad == 0 ? 0 : 1;
}
