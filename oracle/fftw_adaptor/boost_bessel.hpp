/*
 * boost_bessel.hpp -- stand-in for <boost/math/special_functions/bessel.hpp>.
 *
 * TEST INFRASTRUCTURE (oracle only).  The reference calls only
 * boost::math::cyl_bessel_i(0, x) (Reco.h:238-240, Boost 1.66.0).  It is
 * forwarded to the C++17 standard library's std::cyl_bessel_i, which computes
 * the same modified Bessel function of the first kind.  The header is
 * force-included before the reference sources because Reco.h uses the name
 * before Reco.cpp:7 includes Boost.
 */
#pragma once
#include <cmath>
namespace boost { namespace math {
template <class T1, class T2>
inline double cyl_bessel_i(T1 v, T2 x) { return std::cyl_bessel_i((double)v, (double)x); }
} }
