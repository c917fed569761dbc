// abs_overloads.h -- forced include for compiling the reference's bvh_analyzer
// tool (TEST INFRASTRUCTURE ONLY; see ref_harness.cpp).  Its float3.h calls
// unqualified abs() on floats, which libstdc++ resolves to int abs(int); the
// tool was written against MSVC, whose global abs has float overloads.  This
// brings std::abs's overloads into the global scope before the tool's headers
// are read, without changing the reference sources.
#pragma once
#include <cmath>
#include <cstdlib>
using std::abs;
