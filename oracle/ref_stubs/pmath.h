/* Stand-in for the header the reference's math/noise.h includes but does not ship
 * (it comes with the reference's external math library): only what noise.h and
 * noise.cpp use -- the export macro and the C math functions.  Test
 * infrastructure of the oracle's pin to the reference (oracle/ref_build.py). */
#ifndef PMATH_STUB_H
#define PMATH_STUB_H
#include <cmath>
#include <cstdlib>
#ifndef PROLAND_API
#define PROLAND_API
#endif
#endif
