"""The C ABI library: it loads, exports every entry point the header declares and validates its
arguments before touching a device (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from horses3d_gb300 import _abi
from horses3d_gb300.control import Config, UnsupportedOption, parse_control
from horses3d_gb300.mesh import HexMesh

HEADER = Path(__file__).resolve().parents[1] / "include" / "horses3d_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|void|double|int64_t|const char\*)\s+\**(\w+)\s*\(", text)))


def test_header_and_python_signatures_agree():
    names = declared_functions()
    assert "dg_create" in names and "dg_rk3_step" in names and "h3d_mesh_box" in names
    assert sorted(n for n, _, _ in _abi.SIGNATURES) == names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(_abi.library_path()))
    for name in declared_functions():
        assert hasattr(lib, name), name
    L = _abi.lib()
    assert b"sm_103a" in L.dg_version()
    assert L.dg_strerror(_abi.DG_ERR_NAN) == b"NaN or Inf in the solution"


def _ctx_create(mesh, cfg):
    h = C.c_void_p()
    rc = _abi.lib().dg_create(C.byref(mesh.desc), C.byref(cfg.physics()), C.byref(cfg.options()), C.byref(h))
    if rc == _abi.DG_OK:
        _abi.lib().dg_destroy(h)
    return rc


def test_create_validates_before_touching_the_device():
    mesh = HexMesh.box(2, [0, 0, 0], [1, 1, 1], 3, node_type=_abi.DG_NODES_GAUSS)
    # split form needs Gauss-Lobatto nodes
    assert _ctx_create(mesh, Config(inviscid=_abi.DG_INVISCID_SPLIT)) == _abi.DG_ERR_INVALID
    assert _ctx_create(mesh, Config(mach=-1.0)) == _abi.DG_ERR_INVALID
    assert _ctx_create(mesh, Config(riemann=10)) == _abi.DG_ERR_UNSUPPORTED
    assert _ctx_create(mesh, Config(averaging=7)) == _abi.DG_ERR_UNSUPPORTED
    assert _ctx_create(mesh, Config(gradient_variables=3)) == _abi.DG_ERR_UNSUPPORTED
    big = HexMesh.box(1, [0, 0, 0], [1, 1, 1], 8, node_type=_abi.DG_NODES_GAUSS)
    assert _ctx_create(big, Config()) == _abi.DG_ERR_UNSUPPORTED


def test_variable_order_path_validates_before_touching_the_device():
    # anisotropic orders go to the variable-order path (a batch of one case)
    aniso = HexMesh.box(2, [0, 0, 0], [1, 1, 1], np.tile([2, 3, 4], 8), node_type=_abi.DG_NODES_GAUSS)
    # split form needs Gauss-Lobatto nodes here too
    assert _ctx_create(aniso, Config(inviscid=_abi.DG_INVISCID_SPLIT)) == _abi.DG_ERR_INVALID
    assert b"Gauss-Lobatto" in _abi.lib().dg_last_error()
    assert _ctx_create(aniso, Config(mach=0.0)) == _abi.DG_ERR_INVALID
    # a face order that is not the larger of its two sides' orders
    nf = np.ctypeslib.as_array(aniso.desc.face_nf, shape=(2 * aniso.desc.n_faces,))
    saved = nf.copy()
    nf[0] += 1
    try:
        assert _ctx_create(aniso, Config()) == _abi.DG_ERR_INVALID
        assert b"face order" in _abi.lib().dg_last_error()
    finally:
        nf[:] = saved
    # batches: every case validated, shared node type and equations
    L = _abi.lib()
    h = C.c_void_p()
    descs = (_abi.DgMeshDesc * 2)(aniso.desc, aniso.desc)
    phys = (_abi.DgPhysics * 2)(Config().physics(), Config(mach=-1.0).physics())
    assert L.dg_create_batch(2, descs, phys, C.byref(Config().options()), C.byref(h)) == _abi.DG_ERR_INVALID
    assert b"case 1" in L.dg_last_error()
    phys = (_abi.DgPhysics * 2)(Config().physics(), Config(flow="euler").physics())
    assert L.dg_create_batch(2, descs, phys, C.byref(Config().options()), C.byref(h)) == _abi.DG_ERR_UNSUPPORTED
    assert L.dg_create_batch(0, descs, phys, C.byref(Config().options()), C.byref(h)) == _abi.DG_ERR_INVALID
    assert L.dg_batch_size(None) == 0 and L.dg_case_offset(None, 0) == -1


def test_null_arguments_are_rejected():
    L = _abi.lib()
    h = C.c_void_p()
    assert L.dg_create(None, None, None, C.byref(h)) == _abi.DG_ERR_INVALID
    assert L.dg_rhs(None, 0.0) == _abi.DG_ERR_INVALID
    assert L.dg_rk3_step(None, 0.0, 1.0) == _abi.DG_ERR_INVALID
    assert L.dg_upload_state(None, None) == _abi.DG_ERR_INVALID


def test_mesh_builder_rejects_bad_input(tmp_path):
    L = _abi.lib()
    h = C.c_void_p()
    lo = np.zeros(3)
    hi = np.ones(3)
    assert L.h3d_mesh_box(0, 1, 1, _abi.f64ptr(lo), _abi.f64ptr(hi), 0.0, 0, 0, 3, None, C.byref(h)) == _abi.DG_ERR_INVALID
    assert L.h3d_mesh_box(2, 2, 2, _abi.f64ptr(lo), _abi.f64ptr(hi), 0.1, 0, 0, 3, None, C.byref(h)) == _abi.DG_ERR_INVALID
    assert L.h3d_mesh_read_specmesh(str(tmp_path / "missing.mesh").encode(), 0, 3, None, b"", C.byref(h)) == _abi.DG_ERR_IO
    bad = tmp_path / "bad.mesh"
    bad.write_text("8 1 1\n")
    assert L.h3d_mesh_read_specmesh(str(bad).encode(), 0, 3, None, b"", C.byref(h)) == _abi.DG_ERR_IO


def test_non_periodic_mesh_has_boundary_zones(tmp_path):
    m = HexMesh.from_specmesh(_write_single_hex(tmp_path), 2, periodic="")
    assert m.n_faces == 6 and m.n_boundary_faces == 6
    assert sorted(m.zone_names) == ["back", "bottom", "front", "left", "right", "top"]
    # a boundary face without a zone name is an error
    p = tmp_path / "one.mesh"
    p.write_text(p.read_text().replace("front back", "--- back"))
    with pytest.raises(_abi.DgError):
        HexMesh.from_specmesh(p, 2, periodic="")


def _write_single_hex(tmp_path):
    p = tmp_path / "one.mesh"
    nodes = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    lines = ["8 1 1"] + [f"{a} {b} {c}" for a, b, c in nodes] + ["1 2 3 4 5 6 7 8", "0 0 0 0 0 0",
                                                                  "front back bottom right top left"]
    p.write_text("\n".join(lines) + "\n")
    return p


def test_single_periodic_hex_connects_to_itself(tmp_path):
    m = HexMesh.from_specmesh(_write_single_hex(tmp_path), 2, periodic="front:back,bottom:top,left:right")
    assert m.n_elements == 1 and m.n_faces == 3


CONTROL = """
!-- a reduced copy of the keys of the reference's Convergence.control
                          Mesh file name = ../../TestMeshes/UnitCube4x4.mesh
                          Flow equations = "NS"
                             Mach number = 0.3
                         Reynolds number = 10.0
                        Polynomial order = 7
                    Discretization nodes = Gauss
                          Riemann solver = Roe
                  Viscous discretization = BR1
                                     CFL = 0.5
                                    dCFL = 100000.0
                    Number of time steps = 1000000.0
                              Final time = 1.0
#define boundary Front
   type = periodic
   coupled boundary = Back
#end
#define boundary Back
   type = periodic
   coupled boundary = Front
#end
"""


def test_control_file_keys():
    cfg = parse_control(CONTROL)
    assert cfg.order == 7 and cfg.nodes == _abi.DG_NODES_GAUSS and cfg.riemann == _abi.DG_RIEMANN_ROE
    assert cfg.mach == 0.3 and cfg.reynolds == 10.0 and cfg.prandtl == 0.72
    assert cfg.cfl == 0.5 and cfg.dcfl == 1.0e5 and cfg.t_final == 1.0
    assert cfg.periodic == [("front", "back")]
    split = parse_control("inviscid discretization = split-form\naveraging = Pirozzoli\nreynolds number = 1\n")
    assert split.nodes == _abi.DG_NODES_GAUSS_LOBATTO and split.averaging == _abi.DG_AVG_PIROZZOLI
    with pytest.raises(UnsupportedOption):
        parse_control("viscous discretization = BR2\nreynolds number = 1\n")
    with pytest.raises(UnsupportedOption):
        parse_control("riemann solver = hllc\nreynolds number = 1\n")


def test_riemann_and_averaging_keys():
    c = parse_control("riemann solver = Rusanov\naveraging = Kennedy-Gruber\nreynolds number = 1\n")
    assert c.riemann == _abi.DG_RIEMANN_RUSANOV and c.averaging == _abi.DG_AVG_KENNEDY_GRUBER
    c = parse_control("riemann solver = central\naveraging = ducros\nreynolds number = 1\n")
    assert c.riemann == _abi.DG_RIEMANN_CENTRAL and c.averaging == _abi.DG_AVG_DUCROS
    assert parse_control("averaging = morinishi\nreynolds number = 1\n").averaging == _abi.DG_AVG_MORINISHI
    names = {"standard roe": _abi.DG_RIEMANN_STD_ROE, "Roe-Pike": _abi.DG_RIEMANN_ROE_PIKE,
             "low dissipation roe": _abi.DG_RIEMANN_LOW_DISS_ROE, "matrix dissipation": _abi.DG_RIEMANN_MATRIX_DISS,
             "viscous NS": _abi.DG_RIEMANN_VISCOUS_NS, "u-diss": _abi.DG_RIEMANN_U_DISS}
    for k, v in names.items():
        assert parse_control(f"riemann solver = {k}\nreynolds number = 1\n").riemann == v
    for k, v in (("entropy conserving", _abi.DG_AVG_ENTROPY_CONSERVING), ("Chandrasekar", _abi.DG_AVG_CHANDRASEKAR)):
        assert parse_control(f"averaging = {k}\nreynolds number = 1\n").averaging == v
    for k, v in (("state", _abi.DG_GRADVARS_STATE), ("Entropy", _abi.DG_GRADVARS_ENTROPY),
                 ("energy", _abi.DG_GRADVARS_ENERGY)):
        assert parse_control(f"gradient variables = {k}\nreynolds number = 1\n").gradient_variables == v
    with pytest.raises(UnsupportedOption):
        parse_control("gradient variables = primitive\nreynolds number = 1\n")


def test_anisotropic_order_keys(tmp_path):
    ijk = parse_control("polynomial order i = 2\npolynomial order j = 3\npolynomial order k = 4\nreynolds number = 1\n")
    assert ijk.element_orders() == (2, 3, 4)
    with pytest.raises(ValueError):
        parse_control("polynomial order i = 2\nreynolds number = 1\n")
    (tmp_path / "orders.omesh").write_text("3\n1 2 3\n4 5 6\n7 1 2\n")
    f = parse_control("polynomial order = 5\npolynomial order file = orders.omesh\nreynolds number = 1\n")
    assert f.element_orders(tmp_path).tolist() == [[1, 2, 3], [4, 5, 6], [7, 1, 2]]


def test_boundary_blocks_of_a_control_file():
    text = """mach number = 0.3
reynolds number = 200
AOA theta = 0.0
AOA phi = 90.0
#define boundary InnerCylinder
  type = NoSlipWall
#end
#define boundary inlet
  type = Inflow
#end
#define boundary outlet
  type = Outflow
  pressure = 50000
#end
#define boundary hot
  type = NoSlipWall
  wall type (adiabatic/isothermal) = isothermal
  wall temperature = 400
#end
#define boundary bottom
  type = periodic
  coupled boundary = top
#end
"""
    c = parse_control(text)
    assert c.periodic == [("bottom", "top")] and c.aoa_phi == 90.0
    wall = c.boundary("InnerCylinder")
    assert wall.type == _abi.DG_BC_NO_SLIP_WALL and wall.isothermal == 0
    hot = c.boundary("hot")
    assert hot.isothermal == 1 and abs(hot.wall_temperature - 400.0 / (520.0 * 5.0 / 9.0)) < 1e-15
    inflow = c.boundary("inlet")  # the free stream: unit density and speed along z
    assert inflow.type == _abi.DG_BC_INFLOW and abs(inflow.rho - 1.0) < 1e-15 and abs(inflow.w - 1.0) < 1e-12
    assert abs(inflow.p - 1.0 / (1.4 * 0.09)) < 1e-12
    out = c.boundary("outlet")
    ref = c._ref()
    assert out.type == _abi.DG_BC_OUTFLOW and abs(out.pressure - 50000.0 / ref["p"]) < 1e-12
    with pytest.raises(ValueError):
        c.boundary("nowhere")


def test_control_zone_lists_and_steady_state_tolerance():
    """A "#define boundary" line names its zones joined by "__" (GenericBoundaryConditionClass.f90:
    400-456); "convergence tolerance" is a Fortran real (1.d-10) that stops a steady-state run."""
    text = """Flow equations = "Euler"
mach number = 0.5
Convergence tolerance = 1.d-10
Number of time steps = 5000
#define boundary left__right__front__back__bottom__top
   type = Inflow
#end
"""
    cfg = parse_control(text)
    assert cfg.convergence_tolerance == 1e-10 and cfg.n_steps == 5000 and cfg.flow == "euler"
    assert set(cfg.boundaries) == {"left", "right", "front", "back", "bottom", "top"}
    assert all(b["type"] == "inflow" for b in cfg.boundaries.values())
    two = parse_control("reynolds number = 1\n#define boundary InnerCylinder\n type = NoSlipWall\n#end\n"
                        "#define boundary Bottom__Top\n type = FreeSlipWall\n#end\n")
    assert {z: b["type"] for z, b in two.boundaries.items()} == {
        "innercylinder": "noslipwall", "bottom": "freeslipwall", "top": "freeslipwall"}
    assert two.convergence_tolerance is None
