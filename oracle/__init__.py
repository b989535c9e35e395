"""CPU oracle for the GB300 hybrid dealiased convolution -- TEST
INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this package, and only as the checker or the timed
CPU baseline.  The product (``fftwpp_gb300``) never imports it.

* ``oracle.hybrid`` -- numpy restatement of the reference's hybrid
  convolution (parameters, index maps, residue transforms, drivers).
* ``oracle.direct`` -- the reference's O(L^d) direct sums (tests/direct.*).
* ``oracle.ref``    -- ctypes access to the reference itself, compiled by
  oracle/Makefile into oracle/_ref/ where the reference sources exist.
"""
