"""Copies the reference's example ISM-V2 mesh files used as test fixtures (text data, no code):
examples/cgsem-elliptic2d/paraboloid/run/square.mesh (64 elements, boundary curves of degree 5, Dirichlet) and
examples/shallowwater/dipole/run/box.mesh (448 elements, straight sides, no-normal-flow walls).

    python tests/golden/extract_reference_meshes.py /path/to/reference
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = {"square.mesh": "examples/cgsem-elliptic2d/paraboloid/run/square.mesh",
         "box.mesh": "examples/shallowwater/dipole/run/box.mesh"}

if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/extract_reference_meshes.py /path/to/reference")
    ref = sys.argv[1]
    for name, rel in FILES.items():
        shutil.copyfile(os.path.join(ref, rel), os.path.join(HERE, name))
        print(name, os.path.getsize(os.path.join(HERE, name)), "bytes")
