"""Element partitions on the GPU: several partition contexts (dg_create_partition) in one process,
their halo exchange (dg_halo_pack / dg_halo_unpack, the buffers moved by device copies) and the
two-phase stages (dg_partition_stage). Every cut face's flux is evaluated by both partitions from
the same data, so the partitioned right-hand side and RK3 steps must equal the single-context run
bit for bit (plain and mixed, with a shared energy reference), and the plain form must match the
oracle to 1e-12. One GPU holds all partitions here; the multi-GPU exchange itself (NCCL) is the same
exchange function with torch.distributed (horses3d_gb300.partition.dist_exchange), whose host side
is tested with gloo ranks in tests/test_partition.py."""
import ctypes as C

import numpy as np
import pytest

import cases
import oracle
from horses3d_gb300 import _abi
from horses3d_gb300.partition import PartitionSolver, max_time_step, mean_energy, partition_mesh, rhs, rk3_step
from horses3d_gb300.problems import rel_l2
from horses3d_gb300.solver import NavierStokesDG

pytestmark = pytest.mark.gpu

FP64, MIXED = _abi.DG_PRECISION_FP64, _abi.DG_PRECISION_MIXED


def _case(kind, precision):
    if kind == "ns_gl":
        return cases.tgv_case(n=4, order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO, perturbation=0.02, seed=5,
                              precision=precision)
    if kind == "ns_gauss_warped":
        return cases.tgv_case(n=4, order=5, nodes=_abi.DG_NODES_GAUSS, warp=0.1, perturbation=0.02, seed=6,
                              riemann=_abi.DG_RIEMANN_LXF, precision=precision)
    if kind == "split_gl":
        return cases.tgv_case(n=4, order=4, nodes=_abi.DG_NODES_GAUSS_LOBATTO, perturbation=0.01, seed=7,
                              riemann=_abi.DG_RIEMANN_LXF, inviscid=_abi.DG_INVISCID_SPLIT,
                              averaging=_abi.DG_AVG_PIROZZOLI, precision=precision)
    if kind == "euler_vortex":
        return cases.vortex_case(n=4, order=3, precision=precision)
    raise ValueError(kind)


@pytest.mark.parametrize("precision", [FP64, MIXED])
@pytest.mark.parametrize("kind,n_parts", [("ns_gl", 2), ("ns_gauss_warped", 3), ("split_gl", 2), ("euler_vortex", 3)])
def test_partitions_equal_the_single_context(kind, n_parts, precision):
    mesh, cfg, q0 = _case(kind, precision)
    parts = partition_mesh(mesh, n_parts)
    solvers = [PartitionSolver(p, cfg) for p in parts]
    single = NavierStokesDG(mesh, cfg)
    try:
        for s, p in zip(solvers, parts):
            s.set_state(p.local_state(q0))
        single.set_state(q0)
        if precision == MIXED:  # one energy reference for every partition and the single context
            e_ref = mean_energy([(p, p.local_state(q0)) for p in parts])
            for s in solvers:
                s.set_energy_reference(e_ref)
            _abi.check(_abi.lib().dg_set_energy_reference(single._h, e_ref), "dg_set_energy_reference")
        rhs(solvers, 0.0)
        single.compute_time_derivative(0.0)
        qd = single.QDot
        for s, p in zip(solvers, parts):
            assert np.array_equal(s.get(_abi.DG_FIELD_QDOT), p.local_state(qd)), (kind, p.rank)
        t = 0.0
        for _ in range(3):
            dt = max_time_step(solvers, 0.4, 0.4)
            assert dt == single.max_time_step(0.4, 0.4)
            rk3_step(solvers, t, dt)
            single.take_rk3_step(t, dt)
            t += dt
        q = single.Q
        for s, p in zip(solvers, parts):
            assert np.array_equal(s.get(_abi.DG_FIELD_Q), p.local_state(q)), (kind, p.rank)
        if precision == FP64:
            o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
            o.set_state(q0)
            tt = 0.0
            for _ in range(3):
                dt = o.max_dt(0.4, 0.4)
                o.rk3_step(tt, dt)
                tt += dt
            got = np.concatenate([s.get(_abi.DG_FIELD_Q) for s in solvers])
            err = rel_l2(got, o.get(0), mesh.quadrature_weights())
            assert np.all(err <= 1e-12), err
    finally:
        for s in solvers:
            s.close()
        single.close()


def test_partition_entry_points_reject_bad_input():
    mesh, cfg, _ = _case("ns_gl", FP64)
    part = partition_mesh(mesh, 2)[0]
    L = _abi.lib()
    h = C.c_void_p()
    assert L.dg_create_partition(C.byref(part.desc), -1, C.byref(cfg.physics()), C.byref(cfg.options()),
                                 C.byref(h)) == _abi.DG_ERR_INVALID
    # too few ghost elements for the faces' element indices
    assert L.dg_create_partition(C.byref(part.desc), part.n_ghost - 1, C.byref(cfg.physics()),
                                 C.byref(cfg.options()), C.byref(h)) == _abi.DG_ERR_INVALID
    s = PartitionSolver(part, cfg)
    try:
        bad = np.array([6 * part.n_elements], dtype=np.int32)  # a ghost slot cannot be sent
        assert L.dg_halo_set_slots(s._h, 1, _abi.i32ptr(bad), 0, None) == _abi.DG_ERR_INVALID
        assert L.dg_partition_stage(s._h, 3, 0, 0.0, 1e-3) == _abi.DG_ERR_INVALID
        assert L.dg_partition_stage(s._h, 0, 0, 0.0, 0.0) == _abi.DG_ERR_INVALID
    finally:
        s.close()
