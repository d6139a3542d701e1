"""Copy the reference's sample-assembly fixtures here (test
infrastructure).

The reference's sample scripts (tests/components/samples/HSS_*.py,
HMS_*.py, UN_*.py) hand these folders' sampleassembly.xml to
loadFirstHomogeneousScatterer; each folder holds the assembly, the
scatterer file with the kernel, and the unit cell (.xyz) and peak files
(.laz, peaks.py) they name.  Run from anywhere:

    python tests/golden/sampleassemblies/copy_sampleassemblies.py [ROOT]

ROOT (the mcvine/acc source tree) defaults to $MCVINE_ACC_REFERENCE, then
/root/reference.
"""

import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FOLDERS = ("isotropic_sphere", "isotropic_hollowcylinder", "isotropic_box",
           "UN", "Al-simplepowderdiffractionkernel", "Al-E_Q_kernel",
           "Al-constantqekernel")
SUFFIXES = (".xml", ".xyz", ".laz", ".py")


def main(root):
    src = os.path.join(root, "tests", "components", "samples",
                       "sampleassemblies")
    for folder in FOLDERS:
        os.makedirs(os.path.join(HERE, folder), exist_ok=True)
        for name in sorted(os.listdir(os.path.join(src, folder))):
            if name.endswith(SUFFIXES):
                shutil.copyfile(os.path.join(src, folder, name),
                                os.path.join(HERE, folder, name))
                print("copied", folder + "/" + name)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else
         os.environ.get("MCVINE_ACC_REFERENCE", "/root/reference"))
