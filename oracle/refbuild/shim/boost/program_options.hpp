/*
 * ORACLE BUILD SHIM -- test infrastructure only.  Declaration-only stand-in for
 * Boost.Program_options (not installed in this image).  openEMS's tools/global.h names these
 * types in the Global settings class; the harness never parses options.
 */
#ifndef OEMS_SHIM_BOOST_PROGRAM_OPTIONS_HPP
#define OEMS_SHIM_BOOST_PROGRAM_OPTIONS_HPP
/* the real header pulls these in; openEMS sources rely on that */
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>
namespace boost { namespace program_options {
class options_description {};
class variables_map {};
class variable_value {};
} }
#endif
