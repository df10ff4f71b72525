"""GPU parity: the CUDA path through the C ABI against the CPU FP64 oracle on the same inputs.

Tolerances: the plain FP64 form must hold the solution within 1e-12 relative L2 per conserved
variable after the steps (STATE_TOL); a single right-hand side is held to 1e-10 (RHS_TOL) because
QDot is a small difference of O(p0 = 1/(gamma M^2)) flux terms (the Taylor-Green density RHS is
nearly zero), so one rounding difference of an FMA is amplified by that cancellation. The mixed form
must hold the solution within 1e-6 relative L2 (FP32 fluxes, FP64 state and RK accumulation).
"""
import numpy as np
import pytest

import cases
import oracle
from horses3d_gb300 import _abi
from horses3d_gb300.problems import rel_l2
from horses3d_gb300.solver import NavierStokesDG

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-12
RHS_TOL = 1e-10
MIXED_TOL = 1e-6


def _pair(mesh, cfg, q0):
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(q0)
    return o, g


def _check_rhs(mesh, cfg, q0, tol=RHS_TOL, t=0.0):
    o, g = _pair(mesh, cfg, q0)
    ref = o.rhs(t)
    g.compute_time_derivative(t)
    got = g.QDot
    err = rel_l2(got, ref)
    assert np.all(err <= tol), err
    if cfg.flow == "ns":
        for f in (_abi.DG_FIELD_UX, _abi.DG_FIELD_UY, _abi.DG_FIELD_UZ):
            gr = o.get(f)
            e2 = np.max(np.abs(g.get(f) - gr)) / max(np.max(np.abs(gr)), 1e-300)
            assert e2 <= tol, (f, e2)
    return o, g


def _check_steps(mesh, cfg, q0, steps, dt, tol=STATE_TOL):
    o, g = _pair(mesh, cfg, q0)
    t = 0.0
    for _ in range(steps):
        o.rk3_step(t, dt)
        g.take_rk3_step(t, dt)
        t += dt
    w = cases.quadrature_weights(mesh)
    err = rel_l2(g.Q, o.get(0), w)
    assert np.all(err <= tol), err
    return err


@pytest.mark.parametrize("order,nodes", [(3, _abi.DG_NODES_GAUSS_LOBATTO), (2, _abi.DG_NODES_GAUSS),
                                         (5, _abi.DG_NODES_GAUSS), (4, _abi.DG_NODES_GAUSS_LOBATTO)])
def test_rhs_tgv_roe(order, nodes):
    mesh, cfg, q0 = cases.tgv_case(n=3, order=order, nodes=nodes)
    _check_rhs(mesh, cfg, q0)


def test_rhs_curvilinear_lxf_gauss_n5():
    mesh, cfg, q0 = cases.tgv_case(n=3, order=5, nodes=_abi.DG_NODES_GAUSS, riemann=_abi.DG_RIEMANN_LXF, warp=0.1)
    _check_rhs(mesh, cfg, q0)


@pytest.mark.parametrize("averaging", [_abi.DG_AVG_PIROZZOLI, _abi.DG_AVG_STANDARD])
def test_rhs_split_form(averaging):
    mesh, cfg, q0 = cases.tgv_case(n=3, order=4, nodes=_abi.DG_NODES_GAUSS_LOBATTO, riemann=_abi.DG_RIEMANN_LXF,
                                   inviscid=_abi.DG_INVISCID_SPLIT, averaging=averaging, perturbation=0.01, seed=7)
    _check_rhs(mesh, cfg, q0)


def test_rhs_euler_vortex():
    mesh, cfg, q0 = cases.vortex_case(n=3, order=3)
    _check_rhs(mesh, cfg, q0)


def test_rk3_steps_tgv_gl_n3():
    mesh, cfg, q0 = cases.tgv_case(n=4, order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO)
    _check_steps(mesh, cfg, q0, steps=20, dt=2e-3)


def test_rk3_steps_curvilinear_gauss_n5():
    mesh, cfg, q0 = cases.tgv_case(n=3, order=5, nodes=_abi.DG_NODES_GAUSS, riemann=_abi.DG_RIEMANN_LXF, warp=0.1)
    _check_steps(mesh, cfg, q0, steps=10, dt=1e-3)


def test_rk3_steps_split_form():
    mesh, cfg, q0 = cases.tgv_case(n=3, order=4, nodes=_abi.DG_NODES_GAUSS_LOBATTO, riemann=_abi.DG_RIEMANN_LXF,
                                   inviscid=_abi.DG_INVISCID_SPLIT, averaging=_abi.DG_AVG_PIROZZOLI,
                                   perturbation=0.01, seed=3)
    _check_steps(mesh, cfg, q0, steps=10, dt=1e-3)


def test_max_dt_matches_oracle():
    mesh, cfg, q0 = cases.tgv_case(n=3, order=4, nodes=_abi.DG_NODES_GAUSS_LOBATTO, warp=0.0)
    o, g = _pair(mesh, cfg, q0)
    for cfl, dcfl in ((0.4, 0.4), (0.5, 1e5)):
        assert abs(g.max_time_step(cfl, dcfl) - o.max_dt(cfl, dcfl)) <= 1e-15 * o.max_dt(cfl, dcfl)


def test_graph_replay_equals_single_steps():
    mesh, cfg, q0 = cases.tgv_case(n=3, order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO)
    g1 = NavierStokesDG(mesh, cfg)
    g1.set_state(q0)
    t = 0.0
    for _ in range(5):
        g1.take_rk3_step(t, 1e-3)
        t += 1e-3
    g2 = NavierStokesDG(mesh, cfg)
    g2.set_state(q0)
    t_end = g2.run_steps(5, 0.0, dt=1e-3)
    assert abs(t_end - 5e-3) < 1e-15
    assert np.array_equal(g1.Q, g2.Q)
    # CFL mode on the device: same as host-driven MaxTimeStep + RKStep
    g3 = NavierStokesDG(mesh, cfg)
    g3.set_state(q0)
    g4 = NavierStokesDG(mesh, cfg)
    g4.set_state(q0)
    t = 0.0
    for _ in range(4):
        dt = g3.max_time_step(0.4, 0.4)
        g3.take_rk3_step(t, dt)
        t += dt
    t4 = g4.run_steps(4, 0.0, dt=0.0, cfl=0.4, dcfl=0.4)
    assert abs(t4 - t) <= 1e-15 * t
    assert np.array_equal(g3.Q, g4.Q)


def test_convergence_case_on_gpu_reaches_the_reference_goldens():
    """The whole Convergence regression (215 CFL steps, manufactured source) on the GPU."""
    mesh, cfg, q0 = cases.convergence_case()
    g = NavierStokesDG(mesh, cfg)
    g.set_state(q0)
    rep = g.integrate_in_time(t0=0.0, compute_after_steps=True)
    assert rep.iterations == 215
    err, qerr = cases.convergence_errors(mesh, g.Q, g.QDot, rep.time)
    assert cases.ftassert_close(cases.CONVERGENCE_RESIDUALS, rep.residuals), rep.residuals - cases.CONVERGENCE_RESIDUALS
    assert cases.ftassert_close(cases.CONVERGENCE_Q_ERRORS, err), err - cases.CONVERGENCE_Q_ERRORS
    assert cases.ftassert_close(cases.CONVERGENCE_QDOT_ERRORS, qerr), qerr - cases.CONVERGENCE_QDOT_ERRORS


@pytest.mark.parametrize("kind", ["tgv_gl3", "warped_gauss5", "split4"])
def test_mixed_precision_within_1e6(kind):
    if kind == "tgv_gl3":
        mesh, cfg, q0 = cases.tgv_case(n=4, order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO,
                                       precision=_abi.DG_PRECISION_MIXED)
        steps, dt = 20, 2e-3
    elif kind == "warped_gauss5":
        mesh, cfg, q0 = cases.tgv_case(n=3, order=5, nodes=_abi.DG_NODES_GAUSS, riemann=_abi.DG_RIEMANN_LXF, warp=0.1,
                                       precision=_abi.DG_PRECISION_MIXED)
        steps, dt = 10, 1e-3
    else:
        mesh, cfg, q0 = cases.tgv_case(n=3, order=4, nodes=_abi.DG_NODES_GAUSS_LOBATTO, riemann=_abi.DG_RIEMANN_LXF,
                                       inviscid=_abi.DG_INVISCID_SPLIT, averaging=_abi.DG_AVG_PIROZZOLI,
                                       perturbation=0.01, seed=3, precision=_abi.DG_PRECISION_MIXED)
        steps, dt = 10, 1e-3
    _check_steps(mesh, cfg, q0, steps, dt, tol=MIXED_TOL)


def test_nan_is_reported_not_trapped():
    """A NaN in the host-staged state is detected by the residual reduction (checkForNan)."""
    mesh, cfg, q0 = cases.tgv_case(n=2, order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO)
    g = NavierStokesDG(mesh, cfg)
    q = q0.copy()
    q[17] = np.nan
    g.set_state(q)
    g.compute_time_derivative(0.0)
    _, nan = g.compute_max_residuals()
    assert nan
    g.set_state(q0)
    g.compute_time_derivative(0.0)
    res, nan = g.compute_max_residuals()
    assert not nan and np.all(np.isfinite(res))


@pytest.mark.parametrize("nodes,inviscid", [(_abi.DG_NODES_GAUSS, _abi.DG_INVISCID_STANDARD),
                                            (_abi.DG_NODES_GAUSS_LOBATTO, _abi.DG_INVISCID_SPLIT)])
def test_rotated_elements(tmp_path, nodes, inviscid):
    """Faces with non-zero leftIndexes2Right rotations (interior elements in rotated local frames)."""
    mesh, cfg, q0 = cases.rotated_tgv_case(tmp_path / "rot.mesh", 3, nodes=nodes, riemann=_abi.DG_RIEMANN_LXF,
                                           inviscid=inviscid, averaging=_abi.DG_AVG_PIROZZOLI)
    assert np.any(np.ctypeslib.as_array(mesh.desc.face_rotation, shape=(mesh.n_faces,)) != 0)
    _check_rhs(mesh, cfg, q0)
    _check_steps(mesh, cfg, q0, steps=3, dt=2e-3)


@pytest.mark.parametrize("precision", [_abi.DG_PRECISION_FP64, _abi.DG_PRECISION_MIXED])
def test_max_dt_filter_ties_and_high_mach(precision):
    """The CFL reduction estimates every node in FP32 and evaluates the FP64 expressions only near the
    estimated minimum. A uniform state makes every node tie; a supersonic perturbed state has large
    kinetic-to-internal energy ratios; both must still give the oracle's FP64 minimum."""
    mesh, cfg, q0 = cases.tgv_case(n=3, order=4, nodes=_abi.DG_NODES_GAUSS, warp=0.1, precision=precision)
    uniform = np.tile([1.0, 0.3, -0.2, 0.1, 180.0], mesh.ndof)
    fast = q0.reshape(-1, 5).copy()
    fast[:, 1:4] *= 40.0  # |u| ~ 40 against a ~ 10: Mach ~ 4
    fast[:, 4] += 0.5 * np.sum(fast[:, 1:4] ** 2, axis=1) / fast[:, 0]
    for q in (uniform, fast.reshape(-1)):
        o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
        o.set_state(q)
        g = NavierStokesDG(mesh, cfg)
        g.set_state(q)
        for cfl, dcfl in ((0.4, 0.4), (0.5, 1e5), (0.3, 1e-3)):
            ref = o.max_dt(cfl, dcfl)
            # the mixed form keeps the metric terms in FP32, so its FP64 quotients see rounded metrics
            tol = 1e-15 if precision == _abi.DG_PRECISION_FP64 else 1e-6
            assert abs(g.max_time_step(cfl, dcfl) - ref) <= tol * ref, (cfl, dcfl)


SOLVERS = [(_abi.DG_RIEMANN_LXF, _abi.DG_AVG_DUCROS), (_abi.DG_RIEMANN_LXF, _abi.DG_AVG_MORINISHI),
           (_abi.DG_RIEMANN_LXF, _abi.DG_AVG_KENNEDY_GRUBER), (_abi.DG_RIEMANN_CENTRAL, _abi.DG_AVG_STANDARD),
           (_abi.DG_RIEMANN_CENTRAL, _abi.DG_AVG_KENNEDY_GRUBER), (_abi.DG_RIEMANN_RUSANOV, _abi.DG_AVG_STANDARD),
           (_abi.DG_RIEMANN_STD_ROE, _abi.DG_AVG_STANDARD), (_abi.DG_RIEMANN_STD_ROE, _abi.DG_AVG_PIROZZOLI),
           (_abi.DG_RIEMANN_ROE_PIKE, _abi.DG_AVG_KENNEDY_GRUBER), (_abi.DG_RIEMANN_ROE_PIKE, _abi.DG_AVG_MORINISHI),
           (_abi.DG_RIEMANN_LOW_DISS_ROE, _abi.DG_AVG_STANDARD), (_abi.DG_RIEMANN_MATRIX_DISS, _abi.DG_AVG_STANDARD),
           (_abi.DG_RIEMANN_MATRIX_DISS, _abi.DG_AVG_CHANDRASEKAR), (_abi.DG_RIEMANN_VISCOUS_NS, _abi.DG_AVG_PIROZZOLI),
           (_abi.DG_RIEMANN_U_DISS, _abi.DG_AVG_DUCROS), (_abi.DG_RIEMANN_LXF, _abi.DG_AVG_ENTROPY_CONSERVING),
           (_abi.DG_RIEMANN_CENTRAL, _abi.DG_AVG_CHANDRASEKAR)]


@pytest.mark.parametrize("riemann,averaging", SOLVERS)
def test_more_riemann_solvers_and_averages(riemann, averaging):
    """Every Riemann solver and average of RiemannSolvers_NS.f90 beyond Roe/LxF: plain form against the
    oracle (RHS 1e-10, state 1e-12) and mixed form within 1e-6 of it."""
    mesh, cfg, q0 = cases.tgv_case(n=3, order=4, nodes=_abi.DG_NODES_GAUSS, riemann=riemann, averaging=averaging,
                                   warp=0.1, mach=0.3, perturbation=0.02, seed=3)
    _check_rhs(mesh, cfg, q0)
    _check_steps(mesh, cfg, q0, steps=2, dt=2e-3)
    import dataclasses

    mixed = dataclasses.replace(cfg, precision=_abi.DG_PRECISION_MIXED)
    _check_steps(mesh, mixed, q0, steps=2, dt=2e-3, tol=MIXED_TOL)


@pytest.mark.parametrize("averaging", [_abi.DG_AVG_DUCROS, _abi.DG_AVG_MORINISHI, _abi.DG_AVG_KENNEDY_GRUBER,
                                       _abi.DG_AVG_ENTROPY_CONSERVING, _abi.DG_AVG_CHANDRASEKAR])
def test_split_form_two_point_fluxes(averaging):
    """Split form with the Ducros, Morinishi, Kennedy-Gruber, entropy-conserving (Ismail-Roe) and
    Chandrasekar two-point fluxes."""
    mesh, cfg, q0 = cases.tgv_case(n=3, order=4, nodes=_abi.DG_NODES_GAUSS_LOBATTO, riemann=_abi.DG_RIEMANN_LXF,
                                   inviscid=_abi.DG_INVISCID_SPLIT, averaging=averaging, perturbation=0.01, seed=5)
    _check_rhs(mesh, cfg, q0)
    _check_steps(mesh, cfg, q0, steps=2, dt=2e-3)
    import dataclasses

    mixed = dataclasses.replace(cfg, precision=_abi.DG_PRECISION_MIXED)
    _check_steps(mesh, mixed, q0, steps=2, dt=2e-3, tol=MIXED_TOL)


def test_solution_file_restart_continues_the_run(tmp_path):
    """Save the device state after two steps, restart a new context from the file and step on: the
    result equals four uninterrupted steps bit for bit (HexMesh_SaveSolution / LoadSolution)."""
    mesh, cfg, q0 = cases.tgv_case(n=3, order=3, nodes=_abi.DG_NODES_GAUSS, perturbation=0.01, seed=2)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(q0)
    dt = 2e-3
    t = g.run_steps(2, 0.0, dt=dt)
    path = tmp_path / "restart.hsol"
    g.save_solution(path, iteration=2, time=t, gradients=True)
    g.run_steps(2, t, dt=dt)
    h = NavierStokesDG(mesh, cfg)
    h.set_state(q0 * 0 + 1.0)
    it, t2 = h.load_solution(path)
    assert it == 2 and t2 == t
    h.run_steps(2, t2, dt=dt)
    assert np.array_equal(g.Q, h.Q)
    from horses3d_gb300 import solution_file

    hd = solution_file.read_header(path)
    assert hd.file_type == 3 and hd.node_type == 1 and hd.n_elements == mesh.n_elements
    q, grad = solution_file.read(path, mesh.order, gradients=True)
    assert np.all(np.isfinite(grad)) and np.abs(grad).max() > 0


@pytest.mark.parametrize("precision", [_abi.DG_PRECISION_FP64, _abi.DG_PRECISION_MIXED])
def test_lamb_vector_case_on_gpu(precision):
    """NavierStokes/LambVector on the GPU (21 fixed steps to t=0.100001, manufactured source): the
    plain form reaches the reference's L2-error golden (ProblemFile.f90:753-756, tol 1e-7
    relative) and matches the oracle's state to 1e-12; the mixed form is within 1e-6 of it."""
    mesh, cfg, q0 = cases.lamb_vector_case(precision=precision)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(q0)
    rep = g.integrate_in_time(t0=0.0)
    assert rep.iterations == 21 and abs(rep.time - 0.100001) < 1e-15
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    t = 0.0
    for _ in range(20):
        o.rk3_step(t, 0.005)
        t += 0.005
    o.rk3_step(t, 0.100001 - t)
    err = rel_l2(g.Q, o.get(0), cases.quadrature_weights(mesh))
    if precision == _abi.DG_PRECISION_FP64:
        l2 = cases.lamb_vector_l2_error(mesh, g.Q, rep.time)
        assert cases.ftassert_equal(cases.LAMB_VECTOR_L2, l2, 1e-7), l2 - cases.LAMB_VECTOR_L2
        assert np.all(err <= STATE_TOL), err
    else:
        assert np.all(err <= MIXED_TOL), err


def test_lamb_vector_source_on_per_element_orders():
    """The LambVector source on the variable-order kernels (orders 2..5 per element and direction)."""
    orders = cases.random_orders(27, 2, 5, 7)
    mesh = cases.HexMesh.box(3, [0, 0, 0], [cases.TWO_PI] * 3, orders, node_type=_abi.DG_NODES_GAUSS)
    cfg = cases.Config(order=5, nodes=_abi.DG_NODES_GAUSS, mach=0.08, reynolds=1600.0, riemann=_abi.DG_RIEMANN_ROE,
                       source=_abi.DG_SOURCE_MMS_LAMB_VECTOR)
    q0 = cases.problems.mms_lamb_vector_state(mesh.x, 0.0)
    _check_rhs(mesh, cfg, q0, t=0.03)
    _check_steps(mesh, cfg, q0, 5, 0.005)


@pytest.mark.parametrize("variant", ["energy", "entropy"])
def test_convergence_variants_on_gpu_reach_the_reference_goldens(variant):
    """Convergence_energy / Convergence_entropy on the GPU: split form on Gauss-Lobatto nodes with the
    energy or entropy gradient variables (Roe + Pirozzoli, matrix dissipation + Chandrasekar)."""
    mesh, cfg, q0 = cases.convergence_variant_case(variant)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(q0)
    rep = g.integrate_in_time(t0=0.0, compute_after_steps=True)
    assert rep.iterations == 137
    err, qerr = cases.convergence_errors(mesh, g.Q, g.QDot, rep.time)
    gres, gerr, gqerr = cases.CONVERGENCE_VARIANT_GOLDENS[variant]
    assert cases.ftassert_close(gres, rep.residuals), rep.residuals - gres
    assert cases.ftassert_close(gerr, err), err - gerr
    assert cases.ftassert_close(gqerr, qerr), qerr - gqerr


@pytest.mark.parametrize("gv", [_abi.DG_GRADVARS_ENTROPY, _abi.DG_GRADVARS_ENERGY])
@pytest.mark.parametrize("nodes", [_abi.DG_NODES_GAUSS, _abi.DG_NODES_GAUSS_LOBATTO])
def test_gradient_variables(gv, nodes):
    """BR1 with the entropy and energy gradient variables (VariableConversion_NS.f90:211-262,
    Physics_NS.f90:306-414) on a curvilinear mesh: RHS and lifted gradients, steps, mixed form."""
    import dataclasses

    mesh, cfg, q0 = cases.tgv_case(n=3, order=4, nodes=nodes, warp=0.1, mach=0.3, perturbation=0.02, seed=8)
    cfg = dataclasses.replace(cfg, gradient_variables=gv)
    _check_rhs(mesh, cfg, q0)
    _check_steps(mesh, cfg, q0, steps=2, dt=2e-3)
    mixed = dataclasses.replace(cfg, precision=_abi.DG_PRECISION_MIXED)
    _check_steps(mesh, mixed, q0, steps=2, dt=2e-3, tol=MIXED_TOL)


@pytest.mark.parametrize("precision", [_abi.DG_PRECISION_FP64, _abi.DG_PRECISION_MIXED])
@pytest.mark.parametrize("order,nodes", [(3, _abi.DG_NODES_GAUSS), (5, _abi.DG_NODES_GAUSS),
                                         (5, _abi.DG_NODES_GAUSS_LOBATTO)])
def test_integrate_on_device_equals_the_step_loop(precision, order, nodes):
    """dg_integrate (IntegrateInTime on the device, one graph per step with the residual monitor)
    gives the state, time and per-step residuals of the host loop MaxTimeStep + TakeRK3Step +
    ComputeMaxResiduals bit for bit. N = 5 runs the fused monitor (the estimate in the first stage's
    volume kernel, the residual records in the last stage's update)."""
    mesh, cfg, q0 = cases.tgv_case(n=3, order=order, nodes=nodes, perturbation=0.02, seed=12,
                                   precision=precision)
    g1 = NavierStokesDG(mesh, cfg)
    g1.set_state(q0)
    t, hist = 0.0, []
    for _ in range(4):
        dt = g1.max_time_step(0.4, 0.4)
        g1.take_rk3_step(t, dt)
        t += dt
        hist.append(g1.compute_max_residuals()[0])
    g2 = NavierStokesDG(mesh, cfg)
    g2.set_state(q0)
    t2, hist2 = g2.integrate_on_device(4, 0.0, cfl=0.4, dcfl=0.4)
    assert t2 == t
    assert np.array_equal(g1.Q, g2.Q)
    assert np.array_equal(np.array(hist), hist2)
    # the same again (the graph is reused) from a fresh upload
    g2.set_state(q0)
    t3, hist3 = g2.integrate_on_device(4, 0.0, cfl=0.4, dcfl=0.4)
    assert t3 == t and np.array_equal(hist3, hist2)


def test_integrate_on_device_reports_the_first_nan_step():
    mesh, cfg, q0 = cases.tgv_case(n=2, order=2, nodes=_abi.DG_NODES_GAUSS)
    g = NavierStokesDG(mesh, cfg)
    q = q0.copy()
    q[7] = np.nan
    g.set_state(q)
    with pytest.raises(FloatingPointError, match="after step 1"):
        g.integrate_on_device(3, 0.0, dt=1e-3)


@pytest.mark.parametrize("precision", [_abi.DG_PRECISION_FP64, _abi.DG_PRECISION_MIXED])
def test_fused_monitor_reports_the_first_nan_step(precision):
    """N = 5 (the fused residual records): a negative density at one node makes the first step's
    pressures and wave speeds NaN; the device loop reports step 1 (the mixed form refuses a NaN
    upload, so the state itself is finite)."""
    mesh, cfg, q0 = cases.tgv_case(n=2, order=5, nodes=_abi.DG_NODES_GAUSS, precision=precision)
    g = NavierStokesDG(mesh, cfg)
    q = q0.copy()
    q[5 * 7] = -1.0
    g.set_state(q)
    with pytest.raises(FloatingPointError, match="after step 1"):
        g.integrate_on_device(3, 0.0, dt=1e-3)


@pytest.mark.parametrize("test", ["TaylorGreen", "TaylorGreenKEPEC"])
def test_taylor_green_reaches_the_reference_goldens(test):
    """NavierStokes TaylorGreen and Euler TaylorGreenKEPEC on the GPU (FP64, 32^3 elements, N=3):
    through the reference-shaped driver the five residuals (tol 1e-7 on value + 1), the kinetic
    energy (1e-11), its rate and, for the Euler case, the entropy rate (1e-11 on value + 1) equal the
    goldens, and for the NavierStokes case the enstrophy (1e-11) from the lifted gradients of the last
    stage, which the steps keep on request (dg_keep_gradients)."""
    mesh, cfg, q0 = cases.taylor_green_reference_case(test)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(q0)
    if cfg.flow == "ns":
        g.keep_gradients(True)
    rep = g.integrate_in_time(t0=0.0)
    gold = cases.TAYLOR_GREEN_GOLDENS[test]
    assert rep.iterations == cfg.n_steps
    assert cases.ftassert_close(gold["residuals"], rep.residuals, 1e-7), rep.residuals - gold["residuals"]
    q, qdot = g.Q, g.QDot
    if cfg.flow == "ns":
        ke, rate, ens = cases.volume_monitors(mesh, q, qdot, g.get(_abi.DG_FIELD_UX), g.get(_abi.DG_FIELD_UY),
                                              g.get(_abi.DG_FIELD_UZ))
        assert cases.ftassert_equal(gold["enstrophy"], ens, 1e-11), ens - gold["enstrophy"]
    else:
        ke, rate, _ = cases.volume_monitors(mesh, q, qdot)
    assert cases.ftassert_equal(gold["kinetic_energy"], ke, 1e-11), ke - gold["kinetic_energy"]
    assert cases.ftassert_close(gold["kinetic_energy_rate"], rate, 1e-11), rate - gold["kinetic_energy_rate"]
    if "entropy_rate" in gold:
        er = cases.entropy_rate(mesh, q, qdot)
        assert cases.ftassert_close(gold["entropy_rate"], er, 1e-11), er - gold["entropy_rate"]
