"""Makes the test fixtures of this directory from the reference tree (run where it is mounted):

  CylinderNSpol3.mesh.gz  the SpecMesh file of Solver/test/TestMeshes/CylinderNSpol3.mesh (the mesh of
                          the EnergyConservingTest and EntropyConservingTest cases)
  Box27.mesh.gz           Solver/test/TestMeshes/Box27.mesh (the mesh of the Euler UniformFlow case)
  CylinderNSpol3_1elem_y.mesh.gz
                          Solver/test/TestMeshes/CylinderNSpol3_1elem_y.mesh and
  OrdersN2N3N4N5_anisotropy.csv.gz
                          Solver/test/NavierStokes/CylinderDifferentOrders/MESH/OrdersN2N3N4N5_anisotropy.csv
                          (the mesh and per-element orders of the CylinderDifferentOrders case)
  BoxAroundCircle3D_extended_pol3.mesh.gz
                          Solver/test/TestMeshes/BoxAroundCircle3D_extended_pol3.mesh (the Euler
                          BoxAroundCircle and BoxAroundCirclePirozzoli cases)
  CubeWithSphere5.mesh.gz Solver/test/TestMeshes/CubeWithSphere5.mesh (the MeshConsistency component test)
  UnitCube4x4.mesh.gz     Solver/test/TestMeshes/UnitCube4x4.mesh (the NavierStokes Convergence case)
  TaylorGreen8.mesh.gz    Solver/test/TestMeshes/TaylorGreen8.mesh (the NavierStokes LambVector case)
  Nodes_3.hsol.gz         Solver/test/AddOns/horsesConverter/Files/Nodes_3.hsol (a solution file with
                          gradients written by the reference)
  <case>.control.gz       the control files of the cases whose configuration the golden tests check

All gzip-compressed, so that the tests can run those cases where the reference is absent.

Usage: python tests/golden/make_fixtures.py <reference root>   (or set $HORSES3D_REFERENCE)
"""
import gzip
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


FILES = ("Solver/test/TestMeshes/CylinderNSpol3.mesh", "Solver/test/TestMeshes/Box27.mesh",
         "Solver/test/TestMeshes/CylinderNSpol3_1elem_y.mesh",
         "Solver/test/NavierStokes/CylinderDifferentOrders/MESH/OrdersN2N3N4N5_anisotropy.csv",
         "Solver/test/TestMeshes/BoxAroundCircle3D_extended_pol3.mesh",
         "Solver/test/TestMeshes/CubeWithSphere5.mesh",
         "Solver/test/TestMeshes/UnitCube4x4.mesh", "Solver/test/TestMeshes/TaylorGreen8.mesh",
         "Solver/test/AddOns/horsesConverter/Files/Nodes_3.hsol",
         *(f"Solver/test/NavierStokes/{c}/{c}.control"
           for c in ("EnergyConservingTest", "EntropyConservingTest", "Cylinder", "CylinderDucros",
                     "CylinderChandrasekarRoe", "CylinderDifferentOrders")),
         *(f"Solver/test/Euler/{c}/{c}.control" for c in ("BoxAroundCircle", "BoxAroundCirclePirozzoli", "UniformFlow")))


def main(root: str = "") -> None:
    root = root or os.environ.get("HORSES3D_REFERENCE", "")
    if not root:
        sys.exit("usage: make_fixtures.py <reference root>  (or set HORSES3D_REFERENCE)")
    for rel in FILES:
        src = Path(root) / rel
        with gzip.GzipFile(HERE / f"{src.name}.gz", "wb", mtime=0) as fh:
            fh.write(src.read_bytes())


if __name__ == "__main__":
    main(*sys.argv[1:])
