"""acc/components/optics/oo_guide.py: an earlier implementation of the straight /
tapering guide with the constructor of guide.py (name, w1, h1, w2, h2, l,
R0, Qc, alpha, m, W) and the same physics; here it is that guide
(MCV_OP_GUIDE).  The reference's tests of this module (reflectivity formula,
pass-through, tests/components/optics/test_oo_guide.py) run against the oracle
in tests/test_oracle_kats.py."""

from .guide import Guide  # noqa: F401

category = 'optics'
