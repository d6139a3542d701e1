"""Copy the reference's two moderator files here, gzip-compressed (the
example instruments of acc_gb300.instruments read them from this folder).

* source_rot2_cdr_cyl_3x3_20190417.dat: an SNS moderator (section 1 the
  spectrum, section 2 the pulse shapes), read by the reference's VERDI
  instrument (tests/instruments/VERDI/VERDI_base.py:17) and its SNS source
  tests (tests/components/sources/test_SNS_source.py);
* BL20-CY-123D-STS-Min-2G-source_mctal-195_sp.dat: an STS moderator
  (section 0 its seven parameters), read by
  tests/components/sources/test_STS_source.py.

Both live in the reference's tests/components/sources.  Run from anywhere:

    python acc_gb300/data/copy_moderators.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to $MCVINE_ACC_REFERENCE, then /root/reference.
"""

import gzip
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ("source_rot2_cdr_cyl_3x3_20190417.dat",
         "BL20-CY-123D-STS-Min-2G-source_mctal-195_sp.dat")


def main(root):
    src = os.path.join(root, "tests", "components", "sources")
    for name in NAMES:
        with open(os.path.join(src, name), "rb") as f, \
                gzip.GzipFile(os.path.join(HERE, name + ".gz"), "wb",
                              compresslevel=9, mtime=0) as g:
            shutil.copyfileobj(f, g)
        print("copied", name)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else
         os.environ.get("MCVINE_ACC_REFERENCE", "/root/reference"))
