// Stand-in for SDAR's Common/Float.h (not part of the reference tree): the
// reference's changeover functions (src/changeover.hpp) use Float as their
// floating type, which SDAR defines as double.  That header also brings in,
// through SDAR and FDPS, the standard headers and the FDPS integer type that
// src/changeover.hpp uses without including them.
#pragma once
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstdlib>
typedef double Float;
namespace PS {
typedef long long S64;
inline void Abort(int code = -1) { std::abort(); (void)code; }
}  // namespace PS
