"""Makes the test fixtures of this directory from the reference tree (run where it is mounted):

  CylinderNSpol3.mesh.gz  the SpecMesh file of Solver/test/TestMeshes/CylinderNSpol3.mesh (the mesh of
                          the EnergyConservingTest and EntropyConservingTest cases), gzip-compressed,
                          so that the GPU tests can run those cases where the reference is absent.

Usage: python tests/golden/make_fixtures.py [reference root]
"""
import gzip
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def main(root: str = "/root/reference") -> None:
    src = Path(root) / "Solver/test/TestMeshes/CylinderNSpol3.mesh"
    data = src.read_bytes()
    with gzip.GzipFile(HERE / "CylinderNSpol3.mesh.gz", "wb", mtime=0) as fh:
        fh.write(data)


if __name__ == "__main__":
    main(*sys.argv[1:])
