"""Failure detection on the GPU without a GPU fault: the update kernel's bounded mbarrier wait is made
to run out (its barrier expects 16 bytes that no bulk copy delivers; every issued copy completes),
the kernel records the failure in a device flag and leaves, the entry point returns DG_ERR_TIMEOUT,
and the same context keeps working after the state is uploaded again."""
import ctypes as C

import numpy as np
import pytest

import cases
import oracle
from horses3d_gb300 import _abi
from horses3d_gb300.problems import rel_l2
from horses3d_gb300.solver import NavierStokesDG

pytestmark = pytest.mark.gpu


def test_bounded_bulk_copy_wait_reports_timeout_and_context_recovers():
    # N = 5 on one element per CTA: the update kernel stages its blocks by TMA
    mesh, cfg, q0 = cases.tgv_case(n=2, order=5, nodes=_abi.DG_NODES_GAUSS, precision=_abi.DG_PRECISION_MIXED)
    L = _abi.lib()
    g = NavierStokesDG(mesh, cfg)
    g.set_state(q0)
    assert L.dg_inject_fault(g._h, _abi.DG_FAULT_TMA_WAIT) == _abi.DG_OK
    assert L.dg_rk3_step(g._h, 0.0, 1e-3) == _abi.DG_ERR_TIMEOUT
    assert b"bounded wait" in L.dg_last_error()
    assert L.dg_inject_fault(g._h, _abi.DG_FAULT_NONE) == _abi.DG_OK
    g.set_state(q0)
    g.take_rk3_step(0.0, 1e-3)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    o.rk3_step(0.0, 1e-3)
    err = rel_l2(g.Q, o.get(0), mesh.quadrature_weights())
    assert np.all(err <= 1e-6), err
    # the graph-replayed path reports it too
    assert L.dg_inject_fault(g._h, _abi.DG_FAULT_TMA_WAIT) == _abi.DG_OK
    t_end = C.c_double()
    assert L.dg_run_steps(g._h, 1, 0.0, 1e-3, 0.0, 0.0, C.byref(t_end)) == _abi.DG_ERR_TIMEOUT
    assert L.dg_inject_fault(g._h, _abi.DG_FAULT_NONE) == _abi.DG_OK
