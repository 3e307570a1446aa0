// HAMeRS_config.hpp as the reference's CMake would generate it from include/HAMeRS_config.hpp.in
// with its default options (CMakeLists.txt:14,45-47: SIMD on, assertion checks on), except that
// std:: smart pointers stand in for Boost's (HAMERS_USE_BOOST off; the same semantics).
#ifndef HAMERS_CONFIG_HPP
#define HAMERS_CONFIG_HPP

#include "SAMRAI/SAMRAI_config.h"

#include <cfloat>

#define HAMERS_ENABLE_SIMD
#define HAMERS_DEBUG_CHECK_ASSERTIONS
#define HAMERS_DEBUG_CHECK_DEV_ASSERTIONS
#define HAMERS_EPSILON 1.0e-15
#define HAMERS_REAL_EPSILON DBL_EPSILON

#endif /* HAMERS_CONFIG_HPP */
