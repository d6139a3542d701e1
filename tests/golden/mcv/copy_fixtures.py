"""Copy the reference's neutron storage fixtures here.

tests/components/sources/singletestneutron.mcv and singletestneutron2.mcv
of the reference were written by mcni's neutron storage
(tests/components/sources/create_neutron_storage_for_test.py): one neutron
each, r=(0,1,2) v=(3,4,5) s=(6,7) t=8 p=9, and r=0 v=(0,0,1000) s=0 t=0
p=1.  They pin the .mcv layout that acc_gb300.neutron_storage reads and
writes.  Run from anywhere: python tests/golden/mcv/copy_fixtures.py
[reference root]; the root defaults to $MCVINE_ACC_REFERENCE, then
/root/reference.
"""

import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ("singletestneutron.mcv", "singletestneutron2.mcv")


def main(root=None):
    root = root or os.environ.get("MCVINE_ACC_REFERENCE", "/root/reference")
    src = os.path.join(root, "tests", "components", "sources")
    for name in NAMES:
        shutil.copyfile(os.path.join(src, name), os.path.join(HERE, name))
        print("copied", name)


if __name__ == "__main__":
    main(*sys.argv[1:])
