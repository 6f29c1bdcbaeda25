/* Minimal stand-in for NeoPZ's TPZTensor.h: only the component enumeration
 * the reference headers use (Voigt order XX, XY, XZ, YY, YZ, ZZ). */
#ifndef ORC_SHIM_TPZTENSOR_H
#define ORC_SHIM_TPZTENSOR_H
enum { _XX_ = 0, _XY_ = 1, _XZ_ = 2, _YY_ = 3, _YZ_ = 4, _ZZ_ = 5 };
#endif
