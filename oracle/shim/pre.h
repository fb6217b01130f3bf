/*
 * pre.h -- force-included ahead of every reference translation unit when the
 * reference is compiled as the CPU oracle (oracle/Makefile).  It changes no
 * reference file; it only supplies what the MSVC build environment provided:
 *  - the standard headers the real Boost header pulled in transitively;
 *  - <math.h> in C++ mode, so unqualified sqrt/abs/fabs/cos/sin on floats pick
 *    the float overloads (as with MSVC's <cmath>);
 *  - std::powf, which MSVC provides and libstdc++ does not (Simulator.cpp:277);
 *  - the MSVC identity high_resolution_clock == steady_clock (Timer.h:15,40);
 *  - public access to private members, so the harness can set ORCA's
 *    neighbour count and time horizons and read component arrays.
 */
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <queue>
#include <random>
#include <stack>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>
#include <math.h>
namespace std { using ::powf; }
#define high_resolution_clock steady_clock
#define private public
