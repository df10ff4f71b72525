"""Properties of every Riemann solver and average of the oracle (no GPU): free-stream preservation on
a curvilinear mesh and discrete conservation on a periodic one."""
import numpy as np
import pytest

import cases
import oracle
from horses3d_gb300 import _abi
from horses3d_gb300.mesh import HexMesh

ALL_RIEMANN = [_abi.DG_RIEMANN_ROE, _abi.DG_RIEMANN_LXF, _abi.DG_RIEMANN_CENTRAL, _abi.DG_RIEMANN_RUSANOV,
               _abi.DG_RIEMANN_STD_ROE, _abi.DG_RIEMANN_ROE_PIKE, _abi.DG_RIEMANN_LOW_DISS_ROE,
               _abi.DG_RIEMANN_MATRIX_DISS, _abi.DG_RIEMANN_VISCOUS_NS, _abi.DG_RIEMANN_U_DISS]
ALL_AVERAGES = [_abi.DG_AVG_STANDARD, _abi.DG_AVG_PIROZZOLI, _abi.DG_AVG_DUCROS, _abi.DG_AVG_MORINISHI,
                _abi.DG_AVG_KENNEDY_GRUBER, _abi.DG_AVG_ENTROPY_CONSERVING, _abi.DG_AVG_CHANDRASEKAR]


def _warped():
    return HexMesh.box(2, [0, 0, 0], [2 * np.pi] * 3, 4, node_type=_abi.DG_NODES_GAUSS, warp=0.1, patch_order=4)


@pytest.mark.parametrize("riemann", ALL_RIEMANN)
def test_every_solver_preserves_a_uniform_flow(riemann):
    """A uniform state has zero right-hand side: every numerical flux is consistent (F*(Q, Q) = F(Q).n)
    and the metric terms are discretely free-stream preserving."""
    mesh = _warped()
    cfg = cases.Config(order=4, nodes=_abi.DG_NODES_GAUSS, mach=0.3, reynolds=100.0, riemann=riemann,
                       averaging=_abi.DG_AVG_CHANDRASEKAR if riemann == _abi.DG_RIEMANN_MATRIX_DISS else 0)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    q = np.tile([1.2, 0.3 * 1.2, -0.2 * 1.2, 0.1 * 1.2, 1.0 / (0.4 * 1.4 * 0.09) + 0.5 * 1.2 * 0.14],
                mesh.ndof)
    o.set_state(q)
    assert np.max(np.abs(o.rhs(0.0))) < 1e-9


@pytest.mark.parametrize("averaging", ALL_AVERAGES)
@pytest.mark.parametrize("inviscid", [_abi.DG_INVISCID_STANDARD, _abi.DG_INVISCID_SPLIT])
def test_every_average_conserves_mass_momentum_energy(averaging, inviscid):
    """On a periodic mesh sum_nodes w J QDot = 0 for every conserved variable: the face fluxes are
    single-valued and the volume terms telescope (standard and split form)."""
    if inviscid == _abi.DG_INVISCID_SPLIT and averaging == _abi.DG_AVG_PIROZZOLI:
        pytest.skip("covered by the split-form parity tests")
    mesh, cfg, q0 = cases.tgv_case(n=2, order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO, riemann=_abi.DG_RIEMANN_LXF,
                                   inviscid=inviscid, averaging=averaging, mach=0.3, perturbation=0.05, seed=4)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    qd = o.rhs(0.0).reshape(-1, 5)
    w = cases.quadrature_weights(mesh)
    total = np.einsum("n,nv->v", w, qd)
    scale = np.einsum("n,nv->v", w, np.abs(qd))
    assert np.all(np.abs(total) <= 1e-12 * scale + 1e-14), total / scale


def test_rest_state_residual_on_nonconforming_curved_faces_is_linear_in_pressure():
    """Where curved faces join elements of different orders the discretisation does not preserve a
    fluid at rest (the two sides' Tset-interpolated metric terms differ); its momentum residual is
    p times a geometry field G. The mixed form relies on that linearity to add p_ref G back."""
    mesh, cfg, _ = cases.aniso_tgv_case(n=3, lo=1, hi=4, seed=41, warp=0.1)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    res = []
    for p in (1.0, 2.0):
        o.set_state(np.tile([1.0, 0.0, 0.0, 0.0, p / 0.4], mesh.ndof))
        res.append(o.rhs(0.0).reshape(-1, 5))
    g1, g2 = res
    assert np.max(np.abs(g1[:, 1:4])) > 1e-3
    assert np.max(np.abs(g2[:, 1:4] - 2.0 * g1[:, 1:4])) <= 1e-12 * np.max(np.abs(g2[:, 1:4]))
    assert np.max(np.abs(g1[:, [0, 4]])) < 1e-12
    straight, cfg2, _ = cases.aniso_tgv_case(n=3, lo=1, hi=4, seed=41, warp=0.0)
    o2 = oracle.Oracle(straight, cfg2.physics(), cfg2.options())
    o2.set_state(np.tile([1.0, 0.0, 0.0, 0.0, 1.0 / 0.4], straight.ndof))
    assert np.max(np.abs(o2.rhs(0.0))) < 1e-11


def _channel(kind_y="noslipwall", n=(3, 2, 2), order=3, nodes=_abi.DG_NODES_GAUSS):
    mesh = HexMesh.box(n, [0, 0, 0], [2.0, 1.0, 1.0], order, node_type=nodes, periodic="left:right,bottom:top")
    cfg = cases.Config(order=order, nodes=nodes, mach=0.3, reynolds=100.0, riemann=_abi.DG_RIEMANN_LXF)
    cfg.boundaries = {"front": {"type": kind_y}, "back": {"type": kind_y}}
    return mesh, cfg


@pytest.mark.parametrize("kind", ["noslipwall", "freeslipwall"])
def test_walls_conserve_mass(kind):
    """A channel with walls at y = 0, 1 (periodic in x and z): the mirrored ghost state carries no
    mass through the walls, so sum w J dRho/dt = 0 for any state."""
    mesh, cfg = _channel(kind)
    assert mesh.n_boundary_faces == 2 * 3 * 2 and sorted(mesh.zone_names) == ["back", "front"]
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options(), cfg.boundary_table(mesh.zone_names))
    rng = np.random.default_rng(3)
    q = np.tile([1.0, 0.3, 0.0, 0.1, 1.0 / (0.4 * 1.4 * 0.09) + 0.05], mesh.ndof).reshape(-1, 5)
    q = q * (1.0 + 0.02 * rng.standard_normal(q.shape))
    o.set_state(q.reshape(-1))
    qd = o.rhs(0.0).reshape(-1, 5)
    w = cases.quadrature_weights(mesh)
    assert abs(np.dot(w, qd[:, 0])) <= 1e-12 * np.dot(w, np.abs(qd[:, 0]))


def test_free_slip_channel_keeps_a_uniform_axial_flow():
    """Uniform flow along x between free-slip walls: the ghost state mirrors a zero normal velocity,
    so the state is steady."""
    mesh, cfg = _channel("freeslipwall")
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options(), cfg.boundary_table(mesh.zone_names))
    o.set_state(np.tile([1.0, 0.4, 0.0, 0.0, 1.0 / (0.4 * 1.4 * 0.09) + 0.08], mesh.ndof))
    assert np.max(np.abs(o.rhs(0.0))) < 1e-10
