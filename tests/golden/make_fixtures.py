"""Makes the test fixtures of this directory from the reference tree (run where it is mounted):

  CylinderNSpol3.mesh.gz  the SpecMesh file of Solver/test/TestMeshes/CylinderNSpol3.mesh (the mesh of
                          the EnergyConservingTest and EntropyConservingTest cases)
  Box27.mesh.gz           Solver/test/TestMeshes/Box27.mesh (the mesh of the Euler UniformFlow case)

Both gzip-compressed, so that the GPU tests can run those cases where the reference is absent.

Usage: python tests/golden/make_fixtures.py [reference root]
"""
import gzip
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


MESHES = ("CylinderNSpol3.mesh", "Box27.mesh")


def main(root: str = "/root/reference") -> None:
    for name in MESHES:
        data = (Path(root) / "Solver/test/TestMeshes" / name).read_bytes()
        with gzip.GzipFile(HERE / f"{name}.gz", "wb", mtime=0) as fh:
            fh.write(data)


if __name__ == "__main__":
    main(*sys.argv[1:])
