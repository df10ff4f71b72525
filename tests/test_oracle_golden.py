"""The CPU oracle against the reference's own golden values (no GPU)."""
from pathlib import Path

import numpy as np
import pytest

import cases
import oracle
from horses3d_gb300 import _abi
from horses3d_gb300.mesh import HexMesh, nodal_storage

REF_MESH = "Solver/test/TestMeshes/UnitCube4x4.mesh"
TGV8_MESH = "Solver/test/TestMeshes/TaylorGreen8.mesh"


def _reference_or_skip(rel, tmp_path):
    path = cases.reference_file(rel, tmp_path)
    if path is None:
        pytest.skip(f"{rel}: no fixture and no reference tree (set ${cases.REFERENCE_ENV})")
    return path


def _run_convergence(mesh, cfg):
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    q0, _ = cases.problems.mms_convergence_state(mesh.x, 0.0)
    o.set_state(q0)
    t, it = 0.0, 0
    eps = np.finfo(float).eps
    while True:  # IntegrateInTime with CorrectDt (TimeIntegrator.f90:737-890,1100-1133)
        dt = o.max_dt(cfg.cfl, cfg.dcfl)
        if t + dt > cfg.t_final:
            dt = cfg.t_final - t
        o.rk3_step(t, dt)
        t += dt
        it += 1
        if t >= cfg.t_final or abs(t - cfg.t_final) <= 100 * eps:
            break
    qdot = o.rhs(t)  # "compute time derivative after timestep = .true."
    res, nan = o.residuals()
    err, qerr = cases.convergence_errors(mesh, o.get(0), qdot, t)
    return it, res, err, qerr, nan


def test_convergence_goldens_generated_mesh():
    mesh, cfg, _ = cases.convergence_case()
    it, res, err, qerr, nan = _run_convergence(mesh, cfg)
    assert not nan
    assert it == 215
    assert cases.ftassert_close(cases.CONVERGENCE_RESIDUALS, res), res - cases.CONVERGENCE_RESIDUALS
    assert cases.ftassert_close(cases.CONVERGENCE_Q_ERRORS, err), err - cases.CONVERGENCE_Q_ERRORS
    assert cases.ftassert_close(cases.CONVERGENCE_QDOT_ERRORS, qerr), qerr - cases.CONVERGENCE_QDOT_ERRORS


@pytest.mark.parametrize("variant", ["energy", "entropy"])
def test_convergence_variant_goldens(variant):
    """Convergence_energy (split form, Pirozzoli, Roe, energy gradient variables) and
    Convergence_entropy (split form, Chandrasekar, matrix dissipation, entropy gradient variables)."""
    mesh, cfg, _ = cases.convergence_variant_case(variant)
    it, res, err, qerr, nan = _run_convergence(mesh, cfg)
    assert not nan
    gres, gerr, gqerr = cases.CONVERGENCE_VARIANT_GOLDENS[variant]
    assert cases.ftassert_close(gres, res), res - gres
    assert cases.ftassert_close(gerr, err), err - gerr
    assert cases.ftassert_close(gqerr, qerr), qerr - gqerr


def test_convergence_goldens_reference_mesh_file(tmp_path):
    _, cfg, _ = cases.convergence_case()
    mesh = HexMesh.from_specmesh(_reference_or_skip(REF_MESH, tmp_path), 7, node_type=_abi.DG_NODES_GAUSS,
                                 periodic="front:back,bottom:top,left:right")
    it, res, err, qerr, nan = _run_convergence(mesh, cfg)
    assert it == 215
    assert cases.ftassert_close(cases.CONVERGENCE_RESIDUALS, res)
    assert cases.ftassert_close(cases.CONVERGENCE_Q_ERRORS, err)
    assert cases.ftassert_close(cases.CONVERGENCE_QDOT_ERRORS, qerr)


def run_lamb_vector(mesh, cfg, q0, rk3_step, get_state):
    """IntegrateInTime with a fixed dt and CorrectDt's final-time clip: 20 steps of 0.005 and one
    of 1e-6 to t=0.100001."""
    t, it = 0.0, 0
    eps = np.finfo(float).eps
    while it < cfg.n_steps:
        dt = cfg.dt if t + cfg.dt <= cfg.t_final else cfg.t_final - t
        rk3_step(t, dt)
        t += dt
        it += 1
        if t >= cfg.t_final or abs(t - cfg.t_final) <= 100 * eps:
            break
    return it, t, cases.lamb_vector_l2_error(mesh, get_state(), t)


def _lamb_vector_on_oracle(mesh):
    _, cfg, _ = cases.lamb_vector_case()
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(cases.problems.mms_lamb_vector_state(mesh.x, 0.0))
    return run_lamb_vector(mesh, cfg, None, o.rk3_step, lambda: o.get(0))


def test_lamb_vector_golden_generated_mesh():
    """NavierStokes/LambVector: the L2 error of the solution at t=0.100001 against the manufactured
    state (ProblemFile.f90:753-756, tol 1e-7 relative)."""
    mesh, _, _ = cases.lamb_vector_case()
    it, t, err = _lamb_vector_on_oracle(mesh)
    assert it == 21 and abs(t - 0.100001) < 1e-15
    assert cases.ftassert_equal(cases.LAMB_VECTOR_L2, err, 1e-7), err - cases.LAMB_VECTOR_L2


def test_lamb_vector_golden_reference_mesh_file(tmp_path):
    mesh = HexMesh.from_specmesh(_reference_or_skip(TGV8_MESH, tmp_path), 5, node_type=_abi.DG_NODES_GAUSS,
                                 periodic="front:back,bottom:top,left:right")
    it, t, err = _lamb_vector_on_oracle(mesh)
    assert it == 21
    assert cases.ftassert_equal(cases.LAMB_VECTOR_L2, err, 1e-7), err - cases.LAMB_VECTOR_L2


CONSERVING_TESTS = "Solver/test/NavierStokes"


@pytest.mark.parametrize("test", ["EnergyConservingTest", "EntropyConservingTest"])
def test_conserving_cylinder_goldens(test, tmp_path):
    """Flow past a cylinder (CylinderNSpol3.mesh, curved N=3 boundary patches) with no-slip walls on
    the cylinder and the side walls, periodic elsewhere: split form (Pirozzoli / Chandrasekar),
    central fluxes, energy / entropy gradient variables, N=5, 10 CFL steps from the free stream.
    The five residuals are the goldens. The reference's own control file (committed fixture) must
    give the same configuration."""
    cfg = cases.conserving_cylinder_config(test)
    control = cases.reference_file(f"{CONSERVING_TESTS}/{test}/{test}.control", tmp_path)
    if control is not None:
        from horses3d_gb300.control import read_control

        rc = read_control(control)
        for k in ("order", "nodes", "mach", "reynolds", "riemann", "inviscid", "averaging", "gradient_variables",
                  "cfl", "dcfl", "n_steps", "aoa_theta", "aoa_phi", "periodic"):
            assert getattr(rc, k) == getattr(cfg, k), k
        assert {z: b["type"] for z, b in rc.boundaries.items()} == {z: b["type"] for z, b in cfg.boundaries.items()}
    mesh = cases.cylinder_mesh(cfg, tmp_path)
    assert mesh.n_boundary_faces == 168 and set(mesh.zone_names) == {"innercylinder", "left", "right"}
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options(), cfg.boundary_table(mesh.zone_names))
    o.set_state(cases.free_stream_state(cfg, mesh))
    t = 0.0
    for _ in range(cfg.n_steps):
        dt = o.max_dt(cfg.cfl, cfg.dcfl)
        o.rk3_step(t, dt)
        t += dt
    o.rhs(t)  # "compute time derivative after timestep = .true."
    res, nan = o.residuals()
    g = cases.CONSERVING_GOLDENS[test]
    assert not nan
    assert cases.ftassert_close(g[[0, 1, 3, 4]], res[[0, 1, 3, 4]], 1e-11), res - g
    assert cases.ftassert_close(g[2], res[2], 1e-10), res - g


CYLINDER_TESTS = "Solver/test/NavierStokes"


@pytest.mark.parametrize("case", ["Cylinder", "CylinderDucros", "CylinderChandrasekarRoe", "CylinderDifferentOrders"])
def test_cylinder_family_goldens(case, tmp_path):
    """Flow past the cylinder with all four boundary kinds (no-slip cylinder, free-slip bottom/top,
    inflow back/left/front, outflow right): standard form with Roe, split form with the Ducros and
    Chandrasekar averages, and per-element anisotropic orders (N 2..5). The five residuals after
    100 CFL steps from the free stream are the goldens. The reference's control file (committed
    fixture) must give the same configuration."""
    cfg = cases.cylinder_case_config(case)
    control = cases.reference_file(f"{CYLINDER_TESTS}/{case}/{case}.control", tmp_path)
    if control is not None:
        from horses3d_gb300.control import read_control

        rc = read_control(control)
        for k in ("nodes", "mach", "reynolds", "prandtl", "riemann", "inviscid", "averaging", "lambda_stab", "cfl",
                  "dcfl", "n_steps", "aoa_theta", "aoa_phi", "periodic", "flow", "gradient_variables", "source"):
            assert getattr(rc, k) == getattr(cfg, k), k
        assert (rc.order_file is None) == (cfg.order_file is None)
        if cfg.order_file is None:
            assert rc.order == cfg.order
        else:
            assert Path(rc.order_file).name == Path(cfg.order_file).name
        assert {z: b["type"] for z, b in rc.boundaries.items()} == {z: b["type"] for z, b in cfg.boundaries.items()}
    mesh = cases.cylinder_case_mesh(case, cfg, tmp_path)
    assert set(mesh.zone_names) == set(cfg.boundaries)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options(), cfg.boundary_table(mesh.zone_names))
    o.set_state(cases.free_stream_state(cfg, mesh))
    t = 0.0
    for _ in range(cfg.n_steps):
        dt = o.max_dt(cfg.cfl, cfg.dcfl)
        o.rk3_step(t, dt)
        t += dt
    res, nan = o.residuals()
    gold, tol = cases.CYLINDER_GOLDENS[case]
    assert not nan
    assert cases.ftassert_close(gold, res, tol), res - gold


EULER_TESTS = "Solver/test/Euler"


@pytest.mark.parametrize("case", ["BoxAroundCircle", "BoxAroundCirclePirozzoli"])
def test_box_around_circle_goldens(case, tmp_path):
    """Euler flow around a cylinder in a box (BoxAroundCircle3D_extended_pol3.mesh, curved N=3
    patches): free-slip walls on the cylinder, bottom and top, inflow on the other four sides,
    standard Roe, standard form or split form with the Pirozzoli average. The five residuals after
    1000 CFL steps (CFL 0.7) from the free stream are the goldens (tol 1e-11 on value + 1)."""
    cfg = cases.box_around_circle_config(case)
    control = cases.reference_file(f"{EULER_TESTS}/{case}/{case}.control", tmp_path)
    if control is not None:
        from horses3d_gb300.control import read_control

        rc = read_control(control)
        for k in ("order", "nodes", "mach", "riemann", "inviscid", "averaging", "lambda_stab", "cfl", "dcfl", "n_steps",
                  "aoa_theta", "aoa_phi", "periodic", "flow", "convergence_tolerance"):
            assert getattr(rc, k) == getattr(cfg, k), k
        assert {z: b["type"] for z, b in rc.boundaries.items()} == {z: b["type"] for z, b in cfg.boundaries.items()}
    mesh = cases.box_around_circle_mesh(cfg, tmp_path)
    assert set(mesh.zone_names) == set(cfg.boundaries)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options(), cfg.boundary_table(mesh.zone_names))
    o.set_state(cases.free_stream_state(cfg, mesh))
    t = 0.0
    for _ in range(cfg.n_steps):
        dt = o.max_dt(cfg.cfl, cfg.dcfl)
        o.rk3_step(t, dt)
        t += dt
    res, nan = o.residuals()
    gold = cases.BOX_AROUND_CIRCLE_GOLDENS[case]
    assert not nan
    assert cases.ftassert_close(gold, res, 1e-11), res - gold


UNIFORM_FLOW = "Solver/test/Euler/UniformFlow"


@pytest.mark.parametrize("order", [3, 4, 5])
def test_uniform_flow_goldens(order, tmp_path):
    """Euler UniformFlow on Box27.mesh: inflow conditions on all six sides, Rusanov, CFL 0.4, M=0.5,
    from the free stream with a 5 % density bump in every element, marched until the maximum
    residual reaches 1e-10 (TimeIntegrator.f90:737-890, steady state). Goldens: the iteration count
    (exact) and the final residual per order (FTAssertEqual, tol 1e-3), and the final state equal to
    the free stream within 1e-10 (ProblemFile.f90:320-372). The reference's
    control file (committed fixture) must give the same configuration."""
    cfg = cases.uniform_flow_config(order)
    control = cases.reference_file(f"{UNIFORM_FLOW}/UniformFlow.control", tmp_path)
    if control is not None:
        from horses3d_gb300.control import read_control

        rc = read_control(control)
        for k in ("nodes", "mach", "riemann", "cfl", "aoa_theta", "aoa_phi", "flow", "n_steps", "convergence_tolerance"):
            assert getattr(rc, k) == getattr(cfg, k), k
        assert rc.order == 5 and rc.periodic == []
        assert {z: b["type"] for z, b in rc.boundaries.items()} == {z: b["type"] for z, b in cfg.boundaries.items()}
    mesh = cases.box27_mesh(cfg, tmp_path)
    assert mesh.n_boundary_faces == 54 and set(mesh.zone_names) == set(cfg.boundaries)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options(), cfg.boundary_table(mesh.zone_names))
    o.set_state(cases.uniform_flow_state(cfg, mesh))
    t, iters, res = 0.0, 0, None
    for k in range(cfg.n_steps):
        dt = o.max_dt(cfg.cfl, cfg.dcfl)
        o.rk3_step(t, dt)
        t += dt
        res, nan = o.residuals()
        assert not nan
        if res.max() <= cfg.convergence_tolerance:
            iters = k + 1
            break
    golden_iters, golden_res = cases.UNIFORM_FLOW_GOLDENS[order]
    assert iters == golden_iters
    assert cases.ftassert_equal(golden_res, res.max(), 1e-3), (res.max(), golden_res)
    err = np.max(np.abs(o.get(0) - cases.free_stream_state(cfg, mesh)))
    assert err <= 1e-10, err


def test_mesh_consistency_cube_with_sphere(tmp_path):
    """MeshConsistencyTests.f90:50-112 (the MeshConsistency component test) on CubeWithSphere5.mesh,
    a 5 x 5 x 5 cube with curved inner elements around a sphere, N=5 Gauss: the quadrature of the
    Jacobian is the volume 125, and the surface of every boundary zone is 25 (tol 1e-13, relative)."""
    import gzip

    path = tmp_path / "CubeWithSphere5.mesh"
    path.write_bytes(gzip.decompress((cases.GOLDEN_DIR / "CubeWithSphere5.mesh.gz").read_bytes()))
    mesh = HexMesh.from_specmesh(path, 5, node_type=_abi.DG_NODES_GAUSS, periodic="")
    vol = float(np.sum(mesh.quadrature_weights()))
    assert cases.ftassert_equal(125.0, vol, 1e-13), vol - 125.0
    assert cases.ftassert_equal(125.0, mesh.volume, 1e-13), mesh.volume - 125.0
    d = mesh.desc
    nf = np.ctypeslib.as_array(d.face_nf, shape=(mesh.n_faces, 2))
    fj = np.ctypeslib.as_array(d.face_jacobian, shape=(mesh.face_points,))
    zone = np.ctypeslib.as_array(d.face_boundary, shape=(mesh.n_faces,))
    surface = np.zeros(len(mesh.zone_names))
    off = 0
    for f in range(mesh.n_faces):
        n1, n2 = int(nf[f, 0]), int(nf[f, 1])
        npt = (n1 + 1) * (n2 + 1)
        if zone[f] >= 0:
            w1 = nodal_storage(_abi.DG_NODES_GAUSS, n1)[1]
            w2 = nodal_storage(_abi.DG_NODES_GAUSS, n2)[1]
            surface[zone[f]] += np.sum(np.outer(w2, w1).ravel() * fj[off:off + npt])
        off += npt
    assert off == mesh.face_points and len(mesh.zone_names) == 6
    for z, s in zip(mesh.zone_names, surface):
        assert cases.ftassert_equal(25.0, s, 1e-13), (z, s - 25.0)


@pytest.mark.parametrize("test", ["TaylorGreen", "TaylorGreenKEPEC"])
def test_taylor_green_goldens(test):
    """NavierStokes TaylorGreen (N=3 Gauss, Roe, BR1, M=0.08, Re=1600, 5 CFL steps) and Euler
    TaylorGreenKEPEC (split form, Chandrasekar, central flux, 10 steps) on a 32^3 periodic box (a
    generated [0, 2 pi]^3 box in place of TaylorGreen32.mesh, which is not in the reference tree).
    Goldens: the five residuals (tol 1e-7 on value + 1), kinetic energy (1e-11), its rate (1e-11 on
    value + 1), and enstrophy (NS, 1e-11) or the entropy rate (Euler, 1e-11 on value + 1), the
    monitors read with the final Q and the QDot and gradients of the last right-hand side."""
    mesh, cfg, q0 = cases.taylor_green_reference_case(test)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    t = 0.0
    for _ in range(cfg.n_steps):
        dt = o.max_dt(cfg.cfl, cfg.dcfl)
        o.rk3_step(t, dt)
        t += dt
    res, nan = o.residuals()
    g = cases.TAYLOR_GREEN_GOLDENS[test]
    assert not nan
    assert cases.ftassert_close(g["residuals"], res, 1e-7), res - g["residuals"]
    q, qdot = o.get(_abi.DG_FIELD_Q), o.get(_abi.DG_FIELD_QDOT)
    if cfg.flow == "ns":
        ke, rate, ens = cases.volume_monitors(mesh, q, qdot, o.get(_abi.DG_FIELD_UX), o.get(_abi.DG_FIELD_UY),
                                              o.get(_abi.DG_FIELD_UZ))
        assert cases.ftassert_equal(g["enstrophy"], ens, 1e-11), ens - g["enstrophy"]
    else:
        ke, rate, _ = cases.volume_monitors(mesh, q, qdot)
        er = cases.entropy_rate(mesh, q, qdot)
        assert cases.ftassert_close(g["entropy_rate"], er, 1e-11), er - g["entropy_rate"]
    assert cases.ftassert_equal(g["kinetic_energy"], ke, 1e-11), ke - g["kinetic_energy"]
    assert cases.ftassert_close(g["kinetic_energy_rate"], rate, 1e-11), rate - g["kinetic_energy_rate"]


def test_nodal_storage_quadrature_and_derivative():
    # Solver/test/Components/NodalStorage/src/NodalStorageTests.f90:10-63 (N=8 Gauss, tol 1e-12)
    x, w, D = nodal_storage(_abi.DG_NODES_GAUSS, 8)
    assert abs(np.sum(x ** 2 * w) - 2.0 / 3.0) <= 1e-12
    assert np.max(np.abs(D @ (x ** 2) - 2.0 * x)) <= 1e-12
    xl, wl, Dl = nodal_storage(_abi.DG_NODES_GAUSS_LOBATTO, 7)
    assert xl[0] == -1.0 and xl[-1] == 1.0
    assert abs(np.sum(wl) - 2.0) <= 1e-14
    # the weights tabulated in the Convergence test (rounded to 15 digits)
    assert np.max(np.abs(wl - cases.WLGL7)) < 1e-14


def test_box_geometry_volume_and_free_stream_metrics():
    for warp, patch in ((0.0, 0), (0.1, 5)):
        m = HexMesh.box(3, [0, 0, 0], [2 * np.pi] * 3, 5, node_type=_abi.DG_NODES_GAUSS, warp=warp, patch_order=patch)
        assert abs(m.volume - (2 * np.pi) ** 3) < 1e-9 * (2 * np.pi) ** 3
        assert m.n_faces == 3 * m.n_elements


def test_oracle_free_stream_preservation_on_warped_mesh():
    """A uniform state has zero right-hand side on a curvilinear mesh (conservative-curl metrics)."""
    mesh = HexMesh.box(2, [0, 0, 0], [2 * np.pi] * 3, 4, node_type=_abi.DG_NODES_GAUSS, warp=0.1, patch_order=4)
    cfg = cases.Config(order=4, nodes=_abi.DG_NODES_GAUSS, mach=0.3, reynolds=100.0, riemann=_abi.DG_RIEMANN_LXF)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    q = np.tile([1.0, 0.3, -0.2, 0.1, 1.0 / (1.4 * 0.4 * 0.09) + 0.5 * 0.14], mesh.ndof)
    o.set_state(q)
    assert np.max(np.abs(o.rhs(0.0))) < 1e-11


def test_rotated_elements_leave_the_rhs_unchanged(tmp_path):
    """A box whose interior elements list their corners in rotated local frames has faces with non-zero
    leftIndexes2Right rotations (MeshTypes.f90:70-107). The right-hand side of the same physical field
    must have the same weighted L2 norm and integral as on the unrotated box, and a uniform state stays
    uniform."""
    mesh, cfg, _ = cases.rotated_tgv_case(tmp_path / "rot.mesh", 3)
    rot = np.ctypeslib.as_array(mesh.desc.face_rotation, shape=(mesh.n_faces,))
    assert len(set(rot.tolist()) - {0}) >= 4
    box = HexMesh.box(4, [0, 0, 0], [cases.TWO_PI] * 3, 3, node_type=_abi.DG_NODES_GAUSS)
    norms = []
    for m in (box, mesh):
        o = oracle.Oracle(m, cfg.physics(), cfg.options())
        o.set_state(cases.problems.taylor_green(m.x, 0.2))
        r = o.rhs(0.0).reshape(-1, 5)
        w = m.quadrature_weights()
        norms.append(np.sqrt(np.einsum("n,nv->v", w, r * r)))
    assert np.allclose(norms[0], norms[1], rtol=1e-12, atol=0.0), norms
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(np.tile([1.0, 0.3, -0.2, 0.1, 45.0], mesh.ndof))
    assert np.max(np.abs(o.rhs(0.0))) < 1e-10
