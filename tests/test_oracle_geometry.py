"""The product's mesh builder against the oracle's own restatement of the reference geometry
(oracle/geometry.cpp: FacePatchClass.f90, TransfiniteMaps3D.f90, MappedGeometry.f90, the face list
of HexMesh.f90) on periodic boxes: straight, and warped with curved face patches. The node
coordinates, the conservative metric terms, the Jacobian, the face list (elements, sides,
rotations) and the face normals, tangents and surface Jacobians must agree to rounding, and so must
the oracle's right-hand side run on either mesh. No GPU."""
import numpy as np
import pytest

import oracle
from horses3d_gb300 import _abi, problems
from horses3d_gb300.control import Config
from horses3d_gb300.mesh import HexMesh

TWO_PI = 2.0 * np.pi
TOL = 1e-13  # relative to each array's largest magnitude: rounding differences only

CASES = [  # (n, order, node type, warp, patch order)
    (3, 3, _abi.DG_NODES_GAUSS_LOBATTO, 0.0, 0),
    (3, 5, _abi.DG_NODES_GAUSS, 0.1, 5),
    (4, 4, _abi.DG_NODES_GAUSS_LOBATTO, 0.1, 4),
    (3, 4, _abi.DG_NODES_GAUSS, 0.15, 2),
]


def _close(a, b, what):
    scale = max(np.max(np.abs(b)), 1e-300)
    err = np.max(np.abs(a - b)) / scale
    assert err <= TOL, f"{what}: {err:.2e}"


@pytest.mark.parametrize("n,order,nodes,warp,patch", CASES)
def test_box_geometry_matches_the_oracle_restatement(n, order, nodes, warp, patch):
    prod = HexMesh.box(n, [0, 0, 0], [TWO_PI] * 3, order, node_type=nodes, warp=warp, patch_order=patch)
    orc = oracle.BoxMesh(n, [0, 0, 0], [TWO_PI] * 3, order, node_type=nodes, warp=warp, patch_order=patch)
    nd = prod.ndof
    assert orc.ndof == nd and orc.n_faces == prod.n_faces == 3 * n ** 3
    for name, count in (("x", 3 * nd), ("ja_xi", 3 * nd), ("ja_eta", 3 * nd), ("ja_zeta", 3 * nd), ("jacobian", nd),
                        ("inv_jacobian", nd)):
        a = np.ctypeslib.as_array(getattr(prod.desc, name), shape=(count,))
        _close(a, orc.array(name, count), name)
    F = prod.n_faces
    for name, count in (("face_elem", 2 * F), ("face_side", 2 * F), ("face_rotation", F), ("face_nf", 2 * F)):
        a = np.ctypeslib.as_array(getattr(prod.desc, name), shape=(count,))
        assert np.array_equal(a, orc.array(name, count)), name
    nfp = F * (order + 1) ** 2
    for name, count in (("face_normal", 3 * nfp), ("face_t1", 3 * nfp), ("face_t2", 3 * nfp),
                        ("face_jacobian", nfp)):
        a = np.ctypeslib.as_array(getattr(prod.desc, name), shape=(count,))
        _close(a, orc.array(name, count), name)


def test_oracle_right_hand_side_is_the_same_on_either_mesh():
    """The whole chain on a warped Gauss box: the oracle's RHS with the product's geometry and with
    its own geometry."""
    args = (3, [0, 0, 0], [TWO_PI] * 3, 4)
    prod = HexMesh.box(*args, node_type=_abi.DG_NODES_GAUSS, warp=0.1, patch_order=4)
    orc = oracle.BoxMesh(*args, node_type=_abi.DG_NODES_GAUSS, warp=0.1, patch_order=4)
    cfg = Config(order=4, nodes=_abi.DG_NODES_GAUSS, mach=0.1, reynolds=1600.0, riemann=_abi.DG_RIEMANN_LXF)
    q0 = problems.taylor_green(prod.x, 0.1)
    out = []
    for mesh in (prod, orc):
        o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
        o.set_state(q0)
        out.append(o.rhs(0.0))
    assert np.all(problems.rel_l2(out[1], out[0]) <= 1e-12)


def test_box_builder_rejects_patches_above_the_order():
    with pytest.raises(ValueError):
        oracle.BoxMesh(3, [0, 0, 0], [1, 1, 1], 3, warp=0.1, patch_order=5)
