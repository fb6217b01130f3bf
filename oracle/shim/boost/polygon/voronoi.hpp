/* Stand-in for Boost.Polygon's voronoi.hpp (Boost 1.82 is not installed).
   The simulator sources only name the diagram type (ECMDataTypes.h:196-201,
   ECM.cpp:16); the diagram itself is built by ECMGenerator.cpp, which the
   oracle build leaves out and replaces with oracle/ref_harness.cpp. */
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include <algorithm>
namespace boost { namespace polygon {
template <class T> struct voronoi_diagram { void clear() {} };
} }
