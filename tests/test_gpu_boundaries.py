"""Non-periodic boundary conditions on the GPU against the oracle, through the C ABI: no-slip and
free-slip walls (adiabatic and isothermal, moving), inflow and outflow, on uniform orders (plain
and mixed form)."""
import dataclasses

import numpy as np
import pytest

import cases
import oracle
from horses3d_gb300 import _abi
from horses3d_gb300.mesh import HexMesh
from horses3d_gb300.problems import rel_l2
from horses3d_gb300.solver import NavierStokesDG

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-12
RHS_TOL = 1e-10
MIXED_TOL = 1e-6


def _state(mesh, mach, seed=0, amp=0.02, u0=(0.3, 0.0, 0.1)):
    rng = np.random.default_rng(seed)
    x = mesh.x
    rho = 1.0 + amp * np.sin(x[:, 0]) * np.cos(x[:, 1] + 0.3) + amp * rng.standard_normal(mesh.ndof) * 0.1
    u = u0[0] + amp * np.cos(x[:, 2])
    v = u0[1] + amp * np.sin(x[:, 0] + x[:, 2])
    w = u0[2] + amp * np.cos(x[:, 1])
    p = 1.0 / (1.4 * mach ** 2) * (1.0 + amp * np.sin(x[:, 1]))
    q = np.stack([rho, rho * u, rho * v, rho * w, p / 0.4 + 0.5 * rho * (u * u + v * v + w * w)], axis=1)
    return q.reshape(-1)


def _channel(y_kind, x_kinds=None, order=3, nodes=_abi.DG_NODES_GAUSS, n=(3, 2, 2), warp=0.0, **bc):
    """[0, 2 pi] x [0, 2 pi] x [0, 2 pi]: walls of y_kind at y = 0, 2 pi; x periodic unless x_kinds
    gives (left, right) conditions; z periodic."""
    periodic = "bottom:top" + ("" if x_kinds else ",left:right")
    mesh = HexMesh.box(n, [0, 0, 0], [2 * np.pi] * 3, order, node_type=nodes, warp=warp,
                       patch_order=order if warp else 0, periodic=periodic)
    cfg = cases.Config(order=order, nodes=nodes, mach=0.3, reynolds=150.0, riemann=_abi.DG_RIEMANN_ROE)
    cfg.boundaries = {"front": dict({"type": y_kind}, **bc), "back": dict({"type": y_kind}, **bc)}
    if x_kinds:
        cfg.boundaries["left"] = {"type": x_kinds[0]}
        cfg.boundaries["right"] = {"type": x_kinds[1]}
    return mesh, cfg


def _pair(mesh, cfg, q0):
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options(), cfg.boundary_table(mesh.zone_names))
    o.set_state(q0)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(q0)
    return o, g


def _check(mesh, cfg, q0, steps=2, dt=1e-3):
    o, g = _pair(mesh, cfg, q0)
    ref = o.rhs(0.0)
    g.compute_time_derivative(0.0)
    err = rel_l2(g.QDot, ref)
    assert np.all(err <= RHS_TOL), err
    if cfg.flow == "ns":
        for f in (_abi.DG_FIELD_UX, _abi.DG_FIELD_UY, _abi.DG_FIELD_UZ):
            gr = o.get(f)
            e2 = np.max(np.abs(g.get(f) - gr)) / max(np.max(np.abs(gr)), 1e-300)
            assert e2 <= RHS_TOL, (f, e2)
    o, g = _pair(mesh, cfg, q0)
    t = 0.0
    for _ in range(steps):
        o.rk3_step(t, dt)
        g.take_rk3_step(t, dt)
        t += dt
    w = cases.quadrature_weights(mesh)
    err = rel_l2(g.Q, o.get(0), w)
    assert np.all(err <= STATE_TOL), err
    mixed = dataclasses.replace(cfg, precision=_abi.DG_PRECISION_MIXED)
    o, gm = _pair(mesh, mixed, q0)
    t = 0.0
    for _ in range(steps):
        o.rk3_step(t, dt)
        gm.take_rk3_step(t, dt)
        t += dt
    err = rel_l2(gm.Q, o.get(0), w)
    assert np.all(err <= MIXED_TOL), err


@pytest.mark.parametrize("nodes", [_abi.DG_NODES_GAUSS, _abi.DG_NODES_GAUSS_LOBATTO])
def test_no_slip_walls(nodes):
    mesh, cfg = _channel("noslipwall", nodes=nodes)
    _check(mesh, cfg, _state(mesh, cfg.mach))


def test_isothermal_moving_no_slip_walls():
    mesh, cfg = _channel("noslipwall", **{"wall type (adiabatic/isothermal)": "isothermal",
                                          "wall temperature": 310.0, "wall velocity": "[0.2, 0.0, -0.1]"})
    _check(mesh, cfg, _state(mesh, cfg.mach, seed=1))


@pytest.mark.parametrize("wt", ["adiabatic", "isothermal"])
def test_free_slip_walls(wt):
    mesh, cfg = _channel("freeslipwall", **{"wall type (adiabatic/isothermal)": wt})
    _check(mesh, cfg, _state(mesh, cfg.mach, seed=2))


@pytest.mark.parametrize("riemann", [_abi.DG_RIEMANN_ROE, _abi.DG_RIEMANN_LXF, _abi.DG_RIEMANN_MATRIX_DISS])
def test_inflow_outflow_channel(riemann):
    mesh, cfg = _channel("noslipwall", x_kinds=("inflow", "outflow"), order=4)
    cfg = dataclasses.replace(cfg, riemann=riemann, aoa_theta=0.0, aoa_phi=0.0)
    _check(mesh, cfg, _state(mesh, cfg.mach, seed=3, u0=(1.0, 0.0, 0.0)))


def test_split_form_walls_entropy_variables():
    mesh, cfg = _channel("noslipwall", nodes=_abi.DG_NODES_GAUSS_LOBATTO, order=4, warp=0.1)
    cfg = dataclasses.replace(cfg, inviscid=_abi.DG_INVISCID_SPLIT, averaging=_abi.DG_AVG_CHANDRASEKAR,
                              riemann=_abi.DG_RIEMANN_CENTRAL, gradient_variables=_abi.DG_GRADVARS_ENTROPY)
    _check(mesh, cfg, _state(mesh, cfg.mach, seed=4))


def test_euler_walls_and_graph_replay():
    """Euler equations between free-slip walls; graph-replayed steps equal single steps bit for bit."""
    mesh, cfg = _channel("freeslipwall", order=3)
    cfg = dataclasses.replace(cfg, flow="euler")
    q0 = _state(mesh, cfg.mach, seed=5)
    _check(mesh, cfg, q0)
    g1 = NavierStokesDG(mesh, cfg)
    g1.set_state(q0)
    for k in range(3):
        g1.take_rk3_step(k * 1e-3, 1e-3)
    g2 = NavierStokesDG(mesh, cfg)
    g2.set_state(q0)
    g2.run_steps(3, 0.0, dt=1e-3)
    assert np.array_equal(g1.Q, g2.Q)


@pytest.mark.parametrize("test", ["EnergyConservingTest", "EntropyConservingTest"])
def test_conserving_cylinder_cases_reach_the_reference_goldens(test, tmp_path):
    """{Energy,Entropy}ConservingTest on the GPU through the reference-shaped driver: the five
    residuals after 10 CFL steps equal the goldens (tol 1e-11 on x+1, 1e-10 for the y-momentum)."""
    cfg = cases.conserving_cylinder_config(test)
    mesh = cases.cylinder_mesh(cfg, tmp_path)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(cases.free_stream_state(cfg, mesh))
    rep = g.integrate_in_time(t0=0.0, compute_after_steps=True)
    assert rep.iterations == 10
    gold = cases.CONSERVING_GOLDENS[test]
    res = rep.residuals
    assert cases.ftassert_close(gold[[0, 1, 3, 4]], res[[0, 1, 3, 4]], 1e-11), res - gold
    assert cases.ftassert_close(gold[2], res[2], 1e-10), res - gold


def _aniso_channel(y_kind, x_kinds=None, seed=21, lo=1, hi=4, warp=0.0, nodes=_abi.DG_NODES_GAUSS, **bc):
    orders = cases.random_orders(27, lo, hi, seed)
    periodic = "bottom:top" + ("" if x_kinds else ",left:right")
    mesh = HexMesh.box(3, [0, 0, 0], [2 * np.pi] * 3, orders, node_type=nodes, warp=warp,
                       patch_order=hi if warp else 0, periodic=periodic)
    cfg = cases.Config(order=hi, nodes=nodes, mach=0.3, reynolds=150.0, riemann=_abi.DG_RIEMANN_LXF)
    cfg.boundaries = {"front": dict({"type": y_kind}, **bc), "back": dict({"type": y_kind}, **bc)}
    if x_kinds:
        cfg.boundaries["left"] = {"type": x_kinds[0]}
        cfg.boundaries["right"] = {"type": x_kinds[1]}
    return mesh, cfg


@pytest.mark.parametrize("warp", [0.0, 0.1])
def test_anisotropic_orders_no_slip_walls(warp):
    """Per-element orders 1..4 between no-slip walls (variable-order kernels; the walls' faces are
    direct faces at their element side's orders); curved interior with warp."""
    mesh, cfg = _aniso_channel("noslipwall", warp=warp)
    _check(mesh, cfg, _state(mesh, cfg.mach, seed=6))


def test_anisotropic_orders_inflow_outflow_isothermal_walls():
    mesh, cfg = _aniso_channel("noslipwall", x_kinds=("inflow", "outflow"), seed=22, lo=2, hi=5,
                               **{"wall type (adiabatic/isothermal)": "isothermal", "wall temperature": 300.0})
    cfg = dataclasses.replace(cfg, aoa_theta=0.0, aoa_phi=0.0, gradient_variables=_abi.DG_GRADVARS_ENERGY)
    _check(mesh, cfg, _state(mesh, cfg.mach, seed=7, u0=(1.0, 0.0, 0.0)))


def test_batch_with_walled_and_periodic_cases():
    """A batch of a walled channel (anisotropic orders) and a periodic TGV box: each case equals the
    oracle run on it alone."""
    from horses3d_gb300.batch import CaseBatch

    m1, c1 = _aniso_channel("freeslipwall", seed=23)
    q1 = _state(m1, c1.mach, seed=8)
    m2, c2, q2 = cases.tgv_case(n=2, order=3, nodes=_abi.DG_NODES_GAUSS, mach=0.3, reynolds=150.0, perturbation=0.01,
                                seed=9, riemann=_abi.DG_RIEMANN_LXF)
    b = CaseBatch([m1, m2], [c1, c2])
    b.set_state([q1, q2])
    dt = 1e-3
    b.set_clock(np.zeros(2), np.full(2, dt))
    b.run_steps(2)
    got = b.get()
    for (m, c, q), g in zip(((m1, c1, q1), (m2, c2, q2)), got):
        o = oracle.Oracle(m, c.physics(), c.options(), c.boundary_table(m.zone_names) if m.n_boundary_faces else None)
        o.set_state(q)
        for s in range(2):
            o.rk3_step(s * dt, dt)
        err = rel_l2(g, o.get(0), cases.quadrature_weights(m))
        assert np.all(err <= STATE_TOL), err


@pytest.mark.parametrize("order", [3, 5])
def test_uniform_flow_reaches_the_reference_goldens(order, tmp_path):
    """Euler UniformFlow on Box27.mesh (inflow on every side, Rusanov, CFL 0.4, M=0.5) on the GPU:
    the steady-state loop stops at the reference's iteration count with its final residual (FTAssertEqual,
    1e-3), and the state is the free stream within 1e-10. The host-driven loop (integrate_in_time) and
    the device loop (dg_integrate) cross the tolerance at the same step."""
    cfg = cases.uniform_flow_config(order)
    mesh = cases.box27_mesh(cfg, tmp_path)
    iters, golden_res = cases.UNIFORM_FLOW_GOLDENS[order]
    g = NavierStokesDG(mesh, cfg)
    g.set_state(cases.uniform_flow_state(cfg, mesh))
    rep = g.integrate_in_time(t0=0.0)
    assert rep.iterations == iters
    assert cases.ftassert_equal(golden_res, np.max(rep.residuals), 1e-3), (np.max(rep.residuals), golden_res)
    assert np.max(np.abs(g.Q - cases.free_stream_state(cfg, mesh))) <= 1e-10
    d = NavierStokesDG(mesh, cfg)
    d.set_state(cases.uniform_flow_state(cfg, mesh))
    _, hist = d.integrate_on_device(iters, cfl=cfg.cfl, dcfl=cfg.dcfl)
    m = hist.max(axis=1)
    assert m[-1] <= cfg.convergence_tolerance and np.all(m[:-1] > cfg.convergence_tolerance)
    assert np.array_equal(d.Q, g.Q)


@pytest.mark.parametrize("case", ["Cylinder", "CylinderDucros", "CylinderChandrasekarRoe", "CylinderDifferentOrders"])
def test_cylinder_family_reaches_the_reference_goldens(case, tmp_path):
    """The NavierStokes Cylinder cases on the GPU (FP64) through the reference-shaped driver: no-slip,
    free-slip, inflow and outflow boundaries together; standard and split forms; per-element
    anisotropic orders (variable-order kernels). The five residuals after 100 CFL steps equal the
    goldens within each case's tolerance on value + 1."""
    cfg = cases.cylinder_case_config(case)
    mesh = cases.cylinder_case_mesh(case, cfg, tmp_path)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(cases.free_stream_state(cfg, mesh))
    rep = g.integrate_in_time(t0=0.0)
    assert rep.iterations == cfg.n_steps
    gold, tol = cases.CYLINDER_GOLDENS[case]
    assert cases.ftassert_close(gold, rep.residuals, tol), rep.residuals - gold


@pytest.mark.parametrize("case", ["BoxAroundCircle", "BoxAroundCirclePirozzoli"])
def test_box_around_circle_reaches_the_reference_goldens(case, tmp_path):
    """Euler BoxAroundCircle (standard form) and BoxAroundCirclePirozzoli (split form) on the GPU
    (FP64): free-slip walls and inflow, 1000 CFL steps; the five residuals equal the goldens within
    1e-11 on value + 1."""
    cfg = cases.box_around_circle_config(case)
    mesh = cases.box_around_circle_mesh(cfg, tmp_path)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(cases.free_stream_state(cfg, mesh))
    rep = g.integrate_in_time(t0=0.0)
    assert rep.iterations == cfg.n_steps
    gold = cases.BOX_AROUND_CIRCLE_GOLDENS[case]
    assert cases.ftassert_close(gold, rep.residuals, 1e-11), rep.residuals - gold
