"""GPU parity of the variable-order / multi-case path against the CPU FP64 oracle.

p-anisotropic meshes: every element draws its own (Nx, Ny, Nz); each face takes the larger order of
its two sides in each direction and the element traces are interpolated to it (and the face fluxes
projected back) with Tset, as FaceClass.f90:281-470,597-703,865-963 do. Batches: several independent
cases in one context, each compared with the oracle run on that case alone. Tolerances as in
test_gpu_parity: 1e-10 for one right-hand side, 1e-12 for the state after RK3 steps, 1e-6 for the
mixed form.
"""
import numpy as np
import pytest

import cases
import oracle
from horses3d_gb300 import _abi, problems
from horses3d_gb300.batch import CaseBatch
from horses3d_gb300.control import Config
from horses3d_gb300.mesh import HexMesh
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


def _check_rhs(mesh, cfg, q0, t=0.0):
    o, g = _pair(mesh, cfg, q0)
    ref = o.rhs(t)
    g.compute_time_derivative(t)
    err = rel_l2(g.QDot, ref)
    assert np.all(err <= RHS_TOL), err
    if cfg.flow == "ns":
        for f in (_abi.DG_FIELD_UX, _abi.DG_FIELD_UY, _abi.DG_FIELD_UZ):
            gr = o.get(f)
            e2 = np.max(np.abs(g.get(f) - gr)) / max(np.max(np.abs(gr)), 1e-300)
            assert e2 <= RHS_TOL, (f, e2)


def _check_steps(mesh, cfg, q0, steps, dt, tol=STATE_TOL):
    o, g = _pair(mesh, cfg, q0)
    t = 0.0
    for _ in range(steps):
        o.rk3_step(t, dt)
        g.take_rk3_step(t, dt)
        t += dt
    err = rel_l2(g.Q, o.get(0), mesh.quadrature_weights())
    assert np.all(err <= tol), err
    return err


def test_anisotropic_mesh_has_nonconforming_orders():
    mesh, _, _ = cases.aniso_tgv_case(n=3)
    assert mesh.uniform_order() is None
    nf = np.ctypeslib.as_array(mesh.desc.face_nf, shape=(mesh.n_faces, 2))
    assert nf.max() == 4 and nf.min() >= 1


@pytest.mark.parametrize("nodes,riemann", [(_abi.DG_NODES_GAUSS, _abi.DG_RIEMANN_ROE),
                                           (_abi.DG_NODES_GAUSS_LOBATTO, _abi.DG_RIEMANN_LXF)])
def test_rhs_anisotropic_ns(nodes, riemann):
    mesh, cfg, q0 = cases.aniso_tgv_case(n=3, nodes=nodes, riemann=riemann)
    _check_rhs(mesh, cfg, q0)


def test_rhs_anisotropic_curvilinear():
    mesh, cfg, q0 = cases.aniso_tgv_case(n=3, lo=2, hi=5, seed=5, warp=0.1, riemann=_abi.DG_RIEMANN_LXF)
    _check_rhs(mesh, cfg, q0)


@pytest.mark.parametrize("averaging", [_abi.DG_AVG_STANDARD, _abi.DG_AVG_PIROZZOLI])
def test_rhs_anisotropic_euler_vortex(averaging):
    mesh, cfg, q0 = cases.aniso_vortex_case(n=3, averaging=averaging)
    _check_rhs(mesh, cfg, q0)


def test_rk3_steps_anisotropic_ns():
    mesh, cfg, q0 = cases.aniso_tgv_case(n=3, lo=2, hi=5, seed=3, warp=0.1)
    _check_steps(mesh, cfg, q0, steps=3, dt=2e-3)


def test_rk3_steps_anisotropic_euler():
    mesh, cfg, q0 = cases.aniso_vortex_case(n=4, lo=1, hi=6, seed=4)
    _check_steps(mesh, cfg, q0, steps=3, dt=5e-3)


def test_max_dt_anisotropic():
    mesh, cfg, q0 = cases.aniso_tgv_case(n=3, lo=1, hi=6, seed=6)
    o, g = _pair(mesh, cfg, q0)
    for cfl, dcfl in ((0.4, 0.4), (0.5, 1e5)):
        ref = o.max_dt(cfl, dcfl)
        assert abs(g.max_time_step(cfl, dcfl) - ref) <= 1e-15 * ref


def test_anisotropic_graph_replay_with_cfl():
    mesh, cfg, q0 = cases.aniso_tgv_case(n=3, seed=8)
    g1 = NavierStokesDG(mesh, cfg)
    g1.set_state(q0)
    t = 0.0
    for _ in range(3):
        dt = g1.max_time_step(0.4, 0.4)
        g1.take_rk3_step(t, dt)
        t += dt
    g2 = NavierStokesDG(mesh, cfg)
    g2.set_state(q0)
    t2 = g2.run_steps(3, 0.0, dt=0.0, cfl=0.4, dcfl=0.4)
    assert abs(t2 - t) <= 1e-15 * t
    assert np.array_equal(g1.Q, g2.Q)


def test_variable_path_equals_uniform_path_on_a_uniform_mesh():
    """A batch of one uniform case runs the variable-order kernels; it must agree with the
    uniform-order kernels to rounding."""
    mesh, cfg, q0 = cases.tgv_case(n=3, order=3, nodes=_abi.DG_NODES_GAUSS, perturbation=0.01, seed=3)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(q0)
    b = CaseBatch([mesh], [cfg])
    b.set_state([q0])
    g.run_steps(2, 0.0, dt=1e-3)
    b.set_clock(0.0, 1e-3)
    b.run_steps(2)
    err = rel_l2(b.get()[0], g.Q, mesh.quadrature_weights())
    assert np.all(err <= STATE_TOL), err


def test_mixed_anisotropic_within_1e6():
    mesh, cfg, q0 = cases.aniso_tgv_case(n=3, lo=2, hi=5, seed=9, precision=_abi.DG_PRECISION_MIXED)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    g = NavierStokesDG(mesh, cfg)
    g.set_state(q0)
    dt = 2e-3
    for s in range(5):
        o.rk3_step(s * dt, dt)
    g.run_steps(5, 0.0, dt=dt)
    err = rel_l2(g.Q, o.get(0), mesh.quadrature_weights())
    assert np.all(err <= MIXED_TOL), err


def _batch_cases(precision=_abi.DG_PRECISION_FP64):
    out = []
    m, c, q = cases.tgv_case(n=3, order=2, nodes=_abi.DG_NODES_GAUSS, mach=0.3, reynolds=400.0, perturbation=0.01,
                             seed=11, precision=precision)
    out.append((m, c, q))
    m, c, q = cases.aniso_tgv_case(n=2, lo=1, hi=4, seed=12, mach=0.6, reynolds=2500.0, precision=precision)
    out.append((m, c, q))
    m = HexMesh.box(4, [-5.0] * 3, [5.0] * 3, 3, node_type=_abi.DG_NODES_GAUSS)
    c = Config(order=3, nodes=_abi.DG_NODES_GAUSS, mach=0.2, reynolds=150.0, precision=precision)
    q = problems.isentropic_vortex(m.x, 0.2, strength=5.0, period=10.0)
    out.append((m, c, q))
    return out


def test_batch_matches_each_case_alone():
    cs = _batch_cases()
    b = CaseBatch([m for m, _, _ in cs], [c for _, c, _ in cs])
    b.set_state([q for _, _, q in cs])
    assert b.n_cases == 3 and b.ndof == sum(m.ndof for m, _, _ in cs)
    dts = b.max_time_steps(0.4, 0.4)
    refs = []
    for k, (m, c, q) in enumerate(cs):
        o = oracle.Oracle(m, c.physics(), c.options())
        o.set_state(q)
        ref_dt = o.max_dt(0.4, 0.4)
        assert abs(dts[k] - ref_dt) <= 1e-15 * ref_dt, (k, dts[k], ref_dt)
        refs.append(o)
    # every case advances with its own fixed dt
    steps = 3
    b.set_clock(np.zeros(3), dts)
    b.run_steps(steps)
    t, dt = b.clock()
    got = b.get()
    res, nan = b.compute_max_residuals()
    assert not nan.any()
    for k, (m, c, q) in enumerate(cs):
        o = refs[k]
        for s in range(steps):
            o.rk3_step(s * dts[k], dts[k])
        assert abs(t[k] - steps * dts[k]) <= 1e-14 * t[k]
        err = rel_l2(got[k], o.get(0), m.quadrature_weights())
        assert np.all(err <= STATE_TOL), (k, err)
        ref_res, _ = o.residuals()
        assert np.allclose(res[k], ref_res, rtol=1e-9, atol=0.0), (k, res[k], ref_res)


def test_batch_cfl_steps_and_mixed_form():
    cs = _batch_cases(precision=_abi.DG_PRECISION_MIXED)
    b = CaseBatch([m for m, _, _ in cs], [c for _, c, _ in cs])
    b.set_state([q for _, _, q in cs])
    b.set_clock(np.zeros(3), np.zeros(3))
    b.run_steps(4, cfl=0.4, dcfl=0.4)
    t, _ = b.clock()
    got = b.get()
    for k, (m, c, q) in enumerate(cs):
        o = oracle.Oracle(m, c.physics(), c.options())
        o.set_state(q)
        tt = 0.0
        for _ in range(4):
            dt = o.max_dt(0.4, 0.4)
            o.rk3_step(tt, dt)
            tt += dt
        assert abs(t[k] - tt) <= 1e-6 * tt, (k, t[k], tt)
        err = rel_l2(got[k], o.get(0), m.quadrature_weights())
        assert np.all(err <= MIXED_TOL), (k, err)


def test_anisotropic_rotated_elements(tmp_path):
    """Per-element orders on elements in rotated local frames: the right side's face dimensions swap
    under the odd rotations and the Tset interpolation runs in the rotated frame."""
    orders = cases.random_orders(64, 1, 4, seed=3)
    mesh, cfg, q0 = cases.rotated_tgv_case(tmp_path / "rot.mesh", orders)
    rot = np.ctypeslib.as_array(mesh.desc.face_rotation, shape=(mesh.n_faces,))
    assert np.any(np.isin(rot, [1, 3, 4, 6]))
    _check_rhs(mesh, cfg, q0)
    _check_steps(mesh, cfg, q0, steps=3, dt=2e-3)


def test_autotune_keeps_results_and_persists(tmp_path, monkeypatch):
    """Item sizes change how elements are grouped into CTAs, never the arithmetic of a node: results
    after autotuning equal those before, bit for bit, and the state is restored by the tuner."""
    monkeypatch.setenv("HORSES3D_GB300_TUNE_FILE", str(tmp_path / "tune.txt"))
    mesh, cfg, q0 = cases.aniso_tgv_case(n=3, lo=1, hi=5, seed=21)
    g1 = NavierStokesDG(mesh, cfg)
    g1.set_state(q0)
    g1.run_steps(2, 0.0, dt=1e-3)
    g2 = NavierStokesDG(mesh, cfg)
    g2.set_state(q0)
    g2.autotune(reps=2)
    assert np.array_equal(g2.Q, q0)
    g2.run_steps(2, 0.0, dt=1e-3)
    assert np.array_equal(g1.Q, g2.Q)
    rows = {tuple(int(v) for v in ln.split()[:3]) for ln in (tmp_path / "tune.txt").read_text().splitlines() if ln.strip()}
    assert {tuple(int(v) + 1 for v in o) for o in mesh.order} <= rows


@pytest.mark.parametrize("riemann,averaging", [(_abi.DG_RIEMANN_RUSANOV, _abi.DG_AVG_STANDARD),
                                               (_abi.DG_RIEMANN_CENTRAL, _abi.DG_AVG_DUCROS),
                                               (_abi.DG_RIEMANN_LXF, _abi.DG_AVG_KENNEDY_GRUBER),
                                               (_abi.DG_RIEMANN_ROE_PIKE, _abi.DG_AVG_ENTROPY_CONSERVING),
                                               (_abi.DG_RIEMANN_MATRIX_DISS, _abi.DG_AVG_STANDARD),
                                               (_abi.DG_RIEMANN_VISCOUS_NS, _abi.DG_AVG_CHANDRASEKAR),
                                               (_abi.DG_RIEMANN_LOW_DISS_ROE, _abi.DG_AVG_PIROZZOLI)])
def test_anisotropic_more_solvers(riemann, averaging):
    mesh, cfg, q0 = cases.aniso_tgv_case(n=3, lo=1, hi=4, seed=31, riemann=riemann)
    import dataclasses

    cfg = dataclasses.replace(cfg, averaging=averaging)
    _check_rhs(mesh, cfg, q0)
    _check_steps(mesh, cfg, q0, steps=2, dt=2e-3)


def test_batch_save_and_restart_one_case(tmp_path):
    """A case of a batch saved to a solution file and loaded into another batch: that case continues
    bit for bit; a file written from the anisotropic case reads back with its per-element orders."""
    cs = _batch_cases()
    b = CaseBatch([m for m, _, _ in cs], [c for _, c, _ in cs])
    b.set_state([q for _, _, q in cs])
    dts = b.max_time_steps(0.4, 0.4)
    b.set_clock(np.zeros(3), dts)
    b.run_steps(2)
    t, _ = b.clock()
    path = tmp_path / "case1.hsol"
    b.save_solution(1, path, iteration=2, time=t[1])
    from horses3d_gb300 import solution_file

    q_file = solution_file.read(path, cs[1][0].order)
    assert np.array_equal(q_file.reshape(-1), b.get()[1])
    b.run_steps(2)
    c2 = CaseBatch([m for m, _, _ in cs], [c for _, c, _ in cs])
    c2.set_state([q for _, _, q in cs])
    it, t1 = c2.load_solution(1, path)
    assert it == 2 and t1 == t[1]
    c2.set_clock(np.array([0.0, t1, 0.0]), dts)
    c2.run_steps(2)
    assert np.array_equal(c2.get()[1], b.get()[1])


@pytest.mark.parametrize("gv", [_abi.DG_GRADVARS_STATE, _abi.DG_GRADVARS_ENTROPY, _abi.DG_GRADVARS_ENERGY])
def test_anisotropic_gradient_variables(gv):
    """State, entropy and energy gradient variables on per-element orders of a curvilinear mesh: the
    BR1 jumps are formed from the face-point states of both sides after the Tset interpolation. The
    mixed form includes the static-pressure residual of this non-free-stream-preserving geometry."""
    import dataclasses

    mesh, cfg, q0 = cases.aniso_tgv_case(n=3, lo=1, hi=4, seed=41, warp=0.1, riemann=_abi.DG_RIEMANN_LXF)
    cfg = dataclasses.replace(cfg, gradient_variables=gv)
    _check_rhs(mesh, cfg, q0)
    _check_steps(mesh, cfg, q0, steps=2, dt=2e-3)
    mixed = dataclasses.replace(cfg, precision=_abi.DG_PRECISION_MIXED)
    _check_steps(mesh, mixed, q0, steps=2, dt=2e-3, tol=MIXED_TOL)


def test_batch_integrate_on_device():
    """dg_batch_integrate: per-case clocks and residual history, state equal to run_steps."""
    cs = _batch_cases()
    b = CaseBatch([m for m, _, _ in cs], [c for _, c, _ in cs])
    b.set_state([q for _, _, q in cs])
    dts = b.max_time_steps(0.4, 0.4)
    b.set_clock(np.zeros(3), dts)
    b.run_steps(3)
    ref = b.get()
    b.set_state([q for _, _, q in cs])
    b.set_clock(np.zeros(3), dts)
    hist = b.integrate_on_device(3)
    t, _ = b.clock()
    assert np.allclose(t, 3 * dts, rtol=1e-14, atol=0)
    for k in range(3):
        assert np.array_equal(b.get()[k], ref[k])
        assert np.all(hist[:, k, :] > 0)
    res, _ = b.compute_max_residuals()
    assert np.array_equal(hist[-1], res)


_ITEM_SIZE_RUN = """
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import cases
from horses3d_gb300 import _abi
from horses3d_gb300.solver import NavierStokesDG
mesh, cfg, q0 = cases.aniso_tgv_case(n=4, lo=3, hi=4, seed=21, precision=_abi.DG_PRECISION_MIXED)
g = NavierStokesDG(mesh, cfg)
g.set_state(q0)
g.run_steps(3, 0.0, dt=1e-3)
np.save(sys.argv[2], g.Q)
"""


def test_update_store_paths_agree_bit_for_bit(tmp_path):
    """kv_update stores G and Q through shared memory as flat arrays for items of up to 256 nodes and
    per node for larger ones; the item size changes only the grouping, so 64-node and 512-node items
    (the tune file fixes them, one process each) give identical states."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    # 64 elements over 8 order triples (4..5 nodes per direction): 512-node items hold several
    # elements (more than 256 nodes), 64-node items one
    mesh, _, _ = cases.aniso_tgv_case(n=4, lo=3, hi=4, seed=21)
    triples = {tuple(int(v) + 1 for v in o) for o in mesh.order}
    assert len(triples) >= 4
    tests_dir = str(Path(__file__).resolve().parent)
    repo = str(Path(__file__).resolve().parent.parent)
    out = {}
    for cap in (64, 512):
        tune = tmp_path / f"tune{cap}.txt"
        # key: px py pz, FP32 (mixed) form, Navier-Stokes, Gauss nodes -> nodes per item
        tune.write_text("".join(f"{px} {py} {pz} 1 1 {_abi.DG_NODES_GAUSS} {cap}\n" for px, py, pz in sorted(triples)))
        env = dict(os.environ, HORSES3D_GB300_TUNE_FILE=str(tune))
        dst = tmp_path / f"q{cap}.npy"
        subprocess.run([sys.executable, "-c", _ITEM_SIZE_RUN, tests_dir, str(dst)], cwd=repo, env=env, check=True,
                       timeout=600)
        out[cap] = np.load(dst)
    assert np.array_equal(out[64], out[512])


# ---- split form on p-anisotropic meshes (HyperbolicSplitForm.f90:64-116 works per direction with
# the element's orders e%Nxyz(1..3)) ----
def _split(cfg, averaging):
    import dataclasses

    return dataclasses.replace(cfg, inviscid=_abi.DG_INVISCID_SPLIT, averaging=averaging)


@pytest.mark.parametrize("averaging", [_abi.DG_AVG_PIROZZOLI, _abi.DG_AVG_CHANDRASEKAR])
def test_split_form_anisotropic_ns(averaging):
    """Taylor-Green on a warped box with per-element orders 1..5 on Gauss-Lobatto nodes, LxF: one
    right-hand side (1e-10, gradients too) and three RK3 steps (1e-12) against the oracle."""
    mesh, cfg, q0 = cases.aniso_tgv_case(n=3, lo=1, hi=5, seed=12, nodes=_abi.DG_NODES_GAUSS_LOBATTO,
                                         riemann=_abi.DG_RIEMANN_LXF, warp=0.1)
    cfg = _split(cfg, averaging)
    _check_rhs(mesh, cfg, q0)
    o, g = _pair(mesh, cfg, q0)
    t, dt = 0.0, 2e-3
    for _ in range(3):
        o.rk3_step(t, dt)
        g.take_rk3_step(t, dt)
        t += dt
    err = rel_l2(g.Q, o.get(0), mesh.quadrature_weights())
    assert np.all(err <= STATE_TOL), err


def test_split_form_anisotropic_euler_and_mixed():
    """Euler vortex with per-element orders 2..6 (Gauss-Lobatto, Pirozzoli): the plain form within
    1e-12 and the mixed form within 1e-6 of the oracle after five steps."""
    for precision, tol in ((_abi.DG_PRECISION_FP64, STATE_TOL), (_abi.DG_PRECISION_MIXED, MIXED_TOL)):
        mesh, cfg, q0 = cases.aniso_vortex_case(n=3, lo=2, hi=6, seed=13, nodes=_abi.DG_NODES_GAUSS_LOBATTO,
                                                precision=precision)
        cfg = _split(cfg, _abi.DG_AVG_PIROZZOLI)
        o, g = _pair(mesh, cfg, q0)
        dt = 5e-3
        for s in range(5):
            o.rk3_step(s * dt, dt)
        g.run_steps(5, 0.0, dt=dt)
        err = rel_l2(g.Q, o.get(0), mesh.quadrature_weights())
        assert np.all(err <= tol), (precision, err)


def test_split_form_needs_gauss_lobatto_nodes():
    mesh, cfg, _ = cases.aniso_tgv_case(n=2, lo=1, hi=3, seed=1, nodes=_abi.DG_NODES_GAUSS)
    with pytest.raises(_abi.DgError, match="Gauss-Lobatto"):
        NavierStokesDG(mesh, _split(cfg, _abi.DG_AVG_PIROZZOLI))
