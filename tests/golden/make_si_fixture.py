"""Reference values of the sine integral Si(x) from mpmath (50 digits).

The reference evaluates Si through NAG's s13adf Chebyshev expansions
(src/s13adf.f90, called from fforma.f90:188); these values pin any Si
implementation to the function itself.  Run: python tests/golden/make_si_fixture.py
"""
import json
import os

import mpmath

mpmath.mp.dps = 50
XS = [1e-6, 0.01, 0.1, 0.5, 1.0, 2.0, 3.5, 3.999, 4.0, 4.001, 5.0, 7.5, 10.0, 15.9,
      16.1, 20.0, 25.0, 30.0, 40.0, 60.0, 100.0, 250.0]
out = {repr(x): mpmath.nstr(mpmath.si(mpmath.mpf(x)), 30) for x in XS}
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "si_values.json")
json.dump({"source": "mpmath.si at 50 digits", "values": out}, open(dst, "w"), indent=1)
print(dst)
