// host_math.h -- host-side arithmetic shared by the engine and its CPU tests.
#pragma once

#include <cmath>

namespace mdgb {

// The smallest double t whose correctly rounded square root exceeds rc.  The
// reference's pair test sqrt(r^2) <= rc (potential.rs:201-204) is then the
// same as r^2 < t for every double r^2 >= 0: sqrt is monotonic and IEEE-exact
// (correctly rounded) on the host and on the GPU alike.
inline double sqrt_cut(double rc) {
    if (!(rc > 0.0) || !std::isfinite(rc)) return rc > 0.0 ? INFINITY : 0.0;
    double t = rc * rc;
    while (t > 0.0 && std::sqrt(t) > rc) t = std::nextafter(t, 0.0);
    while (std::sqrt(t) <= rc) t = std::nextafter(t, INFINITY);
    return t;
}

}  // namespace mdgb
