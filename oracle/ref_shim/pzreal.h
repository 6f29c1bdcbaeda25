/* Minimal stand-in for NeoPZ's pzreal.h, used only to compile the reference's
 * constitutive headers (Functions*.h) into oracle/_ref for golden vectors.
 * `using std::abs` makes abs() on REAL the floating-point absolute value. */
#ifndef ORC_SHIM_PZREAL_H
#define ORC_SHIM_PZREAL_H
#include <cmath>
#include <cstdlib>
#include <math.h>
using std::abs;
typedef double REAL;
#endif
