"""Correctly rounded FP32 fma on the host, for exact checks of FP32 kernels.

a*b of two FP32 numbers is exact in FP64 (48 significant bits); the sum with c
is rounded once to FP64 and then to FP32.  The second rounding can differ from
a single correct rounding only when the FP64 result lies exactly halfway
between two FP32 numbers; those elements are decided from the exact rational
value (ties to even)."""
from fractions import Fraction

import numpy as np


def fma32(a, b, c):
    """correctly rounded FP32 fma of float32 arrays (broadcast together)"""
    a, b, c = np.broadcast_arrays(*(np.asarray(x, np.float32) for x in (a, b, c)))
    shape = a.shape
    a, b, c = (x.ravel() for x in (a, b, c))
    r = a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)
    out = r.astype(np.float32)
    # a FP64 result exactly halfway between two FP32 numbers may hide a
    # double rounding: decide those from the exact value
    lo = np.where(out.astype(np.float64) > r, np.nextafter(out, np.float32(-np.inf)), out)
    hi = np.nextafter(lo, np.float32(np.inf))
    mid = (lo.astype(np.float64) + hi.astype(np.float64)) / 2
    for i in np.nonzero(r == mid)[0]:
        ex = Fraction(float(a[i])) * Fraction(float(b[i])) + Fraction(float(c[i]))
        m = Fraction(float(mid[i]))
        if ex > m:
            out[i] = hi[i]
        elif ex < m:
            out[i] = lo[i]
        else:
            out[i] = lo[i] if (lo[i:i + 1].view(np.int32)[0] & 1) == 0 else hi[i]
    return out.reshape(shape)
