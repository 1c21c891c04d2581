// Shadow of the reference's include/constants.hpp with g = 9.81, so the
// reference hot path can be run with the gravity that the 256^2 parity case
// states. Placed before the reference on the include path by oracle/Makefile.
#pragma once

namespace constants {
inline constexpr double g = 9.81;
inline constexpr double eps = 1e-8;
} // namespace constants
