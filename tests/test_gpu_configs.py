"""GPU parity at the benchmark configurations' own sizes and step counts, against the FP64 oracle.

Every GPU run goes through the C ABI (NavierStokesDG / CaseBatch). Tolerances, relative L2 per
conserved variable with the quadrature weights: the plain FP64 form STATE_TOL = 1e-12, the mixed
form (FP32 fluxes and contractions, FP64 state, RK accumulation, dt and residuals) MIXED_TOL = 1e-6.

  1  Taylor-Green 8^3, N=3 Gauss-Lobatto, standard form, Roe, BR1, M 0.1, Re 1600, CFL 0.4
     recomputed every step (dCFL 0.4), 100 steps
  2  Taylor-Green 16^3, N=4 Gauss-Lobatto, split form (Pirozzoli), LxF, BR1, +-1 % seeded velocity
     perturbation, CFL 0.4 recomputed every step, 200 steps
  3  curvilinear Taylor-Green 32^3 (warp 0.1 sin x sin y sin z, curved N=5 face patches), N=5 Gauss,
     LxF, BR1, fixed dt from CFL 0.4 at t=0: the full mesh for 40 steps (the oracle takes ~1.2 s per
     step on 16 cores, so 40 of the configuration's 100 steps fit the test budget)
  4  p-anisotropic box, orders (Nx,Ny,Nz) i.i.d. uniform {2..7} (seed 4), Euler isentropic vortex
     (strength 5, M 0.5) advected diagonally, LxF, fixed dt from CFL 0.4 at t=0, 500 steps: a 12^3
     sub-box of the configuration's 24^3 (same domain, orders, vortex and step count; the oracle's
     time for the 2.3 M DOF box does not fit the budget)
  5  the 64 seeded independent NS cases in one batch, each with its own CFL 0.4 dt every step,
     200 steps; every case of the batch is advanced on the GPU, the first six are checked one by
     one against the oracle run on each case alone
The oracle runs with every host core for these sizes.
"""
import os

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
MIXED_TOL = 1e-6
TWO_PI = 2.0 * np.pi
FP64, MIXED = _abi.DG_PRECISION_FP64, _abi.DG_PRECISION_MIXED


@pytest.fixture(autouse=True, scope="module")
def all_cores():
    oracle.set_threads(os.cpu_count() or 1)
    yield
    oracle.set_threads(min(8, os.cpu_count() or 1))


def _replace(cfg, **kw):
    import dataclasses

    return dataclasses.replace(cfg, **kw)


def _oracle_cfl_steps(mesh, cfg, q0, steps, cfl):
    """IntegrateInTime's explicit loop on the oracle: MaxTimeStep(cfl, cfl) then TakeRK3Step."""
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    t = 0.0
    for _ in range(steps):
        dt = o.max_dt(cfl, cfl)
        o.rk3_step(t, dt)
        t += dt
    return o.get(0), t


def _gpu_cfl_steps(mesh, cfg, q0, steps, cfl):
    with NavierStokesDG(mesh, cfg) as g:
        g.set_state(q0)
        t = g.run_steps(steps, 0.0, dt=0.0, cfl=cfl, dcfl=cfl)
        return g.Q, t


def _check(got, ref, mesh, tol, what):
    err = rel_l2(got, ref, mesh.quadrature_weights())
    assert np.all(err <= tol), (what, err)
    return err


def test_config1_tgv8_n3_gl_roe_100_cfl_steps():
    mesh = HexMesh.box(8, [0, 0, 0], [TWO_PI] * 3, 3, node_type=_abi.DG_NODES_GAUSS_LOBATTO)
    cfg = Config(order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO, mach=0.1, reynolds=1600.0, riemann=_abi.DG_RIEMANN_ROE)
    q0 = problems.taylor_green(mesh.x, 0.1)
    ref, t_ref = _oracle_cfl_steps(mesh, cfg, q0, 100, 0.4)
    q, t = _gpu_cfl_steps(mesh, _replace(cfg, precision=FP64), q0, 100, 0.4)
    assert abs(t - t_ref) <= 1e-13 * t_ref
    _check(q, ref, mesh, STATE_TOL, "plain")
    q, _ = _gpu_cfl_steps(mesh, _replace(cfg, precision=MIXED), q0, 100, 0.4)
    _check(q, ref, mesh, MIXED_TOL, "mixed")


def test_config2_split16_n4_pirozzoli_200_cfl_steps():
    mesh = HexMesh.box(16, [0, 0, 0], [TWO_PI] * 3, 4, node_type=_abi.DG_NODES_GAUSS_LOBATTO)
    cfg = Config(order=4, nodes=_abi.DG_NODES_GAUSS_LOBATTO, mach=0.1, reynolds=1600.0, riemann=_abi.DG_RIEMANN_LXF,
                 inviscid=_abi.DG_INVISCID_SPLIT, averaging=_abi.DG_AVG_PIROZZOLI)
    q0 = problems.taylor_green(mesh.x, 0.1, perturbation=0.01, seed=2)
    ref, t_ref = _oracle_cfl_steps(mesh, cfg, q0, 200, 0.4)
    q, t = _gpu_cfl_steps(mesh, _replace(cfg, precision=FP64), q0, 200, 0.4)
    assert abs(t - t_ref) <= 1e-13 * t_ref
    _check(q, ref, mesh, STATE_TOL, "plain")
    q, _ = _gpu_cfl_steps(mesh, _replace(cfg, precision=MIXED), q0, 200, 0.4)
    _check(q, ref, mesh, MIXED_TOL, "mixed")


def test_config3_curvilinear32_n5_full_mesh():
    steps = 40
    mesh = HexMesh.box(32, [0, 0, 0], [TWO_PI] * 3, 5, node_type=_abi.DG_NODES_GAUSS, warp=0.1, patch_order=5)
    cfg = Config(order=5, nodes=_abi.DG_NODES_GAUSS, mach=0.1, reynolds=1600.0, riemann=_abi.DG_RIEMANN_LXF)
    q0 = problems.taylor_green(mesh.x, 0.1)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    dt = o.max_dt(0.4, 0.4)
    for s in range(steps):
        o.rk3_step(s * dt, dt)
    ref = o.get(0)
    del o
    # plain, mixed, and the mixed form with the tensor-core gradient contractions
    for precision, tol in ((FP64, STATE_TOL), (MIXED, MIXED_TOL), (_abi.DG_PRECISION_MIXED_TC, MIXED_TOL)):
        with NavierStokesDG(mesh, _replace(cfg, precision=precision)) as g:
            g.set_state(q0)
            if precision == FP64:
                assert abs(g.max_time_step(0.4, 0.4) - dt) <= 1e-15 * dt
            g.run_steps(steps, 0.0, dt=dt)
            _check(g.Q, ref, mesh, tol, precision)


def test_config4_anisotropic_vortex_subbox_500_steps():
    n, steps = 12, 500
    orders = np.random.default_rng(4).integers(2, 8, size=(n ** 3, 3)).astype(np.int32)
    mesh = HexMesh.box(n, [-5.0] * 3, [5.0] * 3, orders, node_type=_abi.DG_NODES_GAUSS)
    cfg = Config(order=7, nodes=_abi.DG_NODES_GAUSS, flow="euler", mach=0.5, riemann=_abi.DG_RIEMANN_LXF)
    q0 = problems.isentropic_vortex(mesh.x, 0.5, strength=5.0, period=10.0)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    dt = o.max_dt(0.4, 0.4)
    for s in range(steps):
        o.rk3_step(s * dt, dt)
    ref = o.get(0)
    for precision, tol in ((FP64, STATE_TOL), (MIXED, MIXED_TOL)):
        with CaseBatch([mesh], [_replace(cfg, precision=precision)]) as b:
            b.set_state([q0])
            b.set_clock(np.zeros(1), np.array([dt]))
            b.run_steps(steps)
            _check(b.get()[0], ref, mesh, tol, precision)


def test_config5_batch64_per_case_200_cfl_steps():
    import bench

    meshes, cfgs, qs, steps = bench.build_secondary("batch64")
    assert len(meshes) == 64 and steps == 200
    checked = 6
    refs = [_oracle_cfl_steps(m, c, q, steps, 0.4) for m, c, q in zip(meshes[:checked], cfgs[:checked], qs[:checked])]
    for precision, tol in ((FP64, STATE_TOL), (MIXED, MIXED_TOL)):
        with CaseBatch(meshes, [_replace(c, precision=precision) for c in cfgs]) as b:
            b.set_state(qs)
            b.set_clock(np.zeros(64), np.zeros(64))
            b.run_steps(steps, cfl=0.4, dcfl=0.4)
            t, _ = b.clock()
            got = b.get()
            for k in range(checked):
                ref, t_ref = refs[k]
                assert abs(t[k] - t_ref) <= (1e-13 if precision == FP64 else 1e-6) * t_ref, (k, t[k], t_ref)
                _check(got[k], ref, meshes[k], tol, (precision, k))
