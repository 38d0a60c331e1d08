/*
 * ORACLE BUILD SHIM -- test infrastructure only.  Declaration-only stand-in for Boost.StringAlgo
 * (not installed in this image).  openEMS's tools/useful.cpp uses boost::split for string
 * parsing helpers that the engine path never calls, so these abort if reached.
 */
#ifndef OEMS_SHIM_BOOST_ALGORITHM_STRING_HPP
#define OEMS_SHIM_BOOST_ALGORITHM_STRING_HPP
#include <string>
#include "ContinuousStructure.h"
namespace boost {
struct oems_shim_any_of {};
inline oems_shim_any_of is_any_of(const std::string&) { return oems_shim_any_of(); }
template <class R, class S>
R& split(R&, S&, oems_shim_any_of) OEMS_SHIM_ABORT
}
#endif
