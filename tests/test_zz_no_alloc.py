"""dg_max_dt_noalloc: the CFL time step for callers that cannot allocate device memory (a host
that hands out all device memory from its own pool, or code running after an allocation freeze).
The entry point takes device pointers to the caller's state and metrics and keeps its only scratch in
a fixed file-scope device array, so its result must equal the allocating dg_max_dt on the same state.
Two calls in a row (a large mesh, then a small one) also show that the shared scratch carries
nothing from one call into the next. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from horses3d_gb300 import _abi
from horses3d_gb300.solver import NavierStokesDG

pytestmark = pytest.mark.gpu

TOL = 1e-15  # the same FP64 arithmetic and an exact min-reduction: equal up to the last bit


def _device(arr, torch):
    return torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64)).cuda()


def _noalloc_dt(mesh, cfg, q, torch, cfl, dcfl, stream=None):
    """stream: a torch.cuda.Stream to run on (None: the default stream)."""
    t = {name: _device(a, torch) for name, a in (
        ("q", q), ("xi", np.ctypeslib.as_array(mesh.desc.ja_xi, shape=(3 * mesh.ndof,))),
        ("eta", np.ctypeslib.as_array(mesh.desc.ja_eta, shape=(3 * mesh.ndof,))),
        ("zeta", np.ctypeslib.as_array(mesh.desc.ja_zeta, shape=(3 * mesh.ndof,))),
        ("jac", mesh.jacobian))}
    torch.cuda.synchronize()
    dt = C.c_double()
    rc = _abi.lib().dg_max_dt_noalloc(t["q"].data_ptr(), t["xi"].data_ptr(), t["eta"].data_ptr(),
                                      t["zeta"].data_ptr(), t["jac"].data_ptr(), mesh.ndof, cfg.order, cfg.nodes,
                                      C.byref(cfg.physics()), cfl, dcfl,
                                      None if stream is None else stream.cuda_stream, C.byref(dt))
    _abi.check(rc, "dg_max_dt_noalloc")
    return dt.value


def test_noalloc_max_dt_matches_the_allocating_entry_point():
    torch = pytest.importorskip("torch")
    big_mesh, big_cfg, big_q = cases.tgv_case(n=6, order=5, nodes=_abi.DG_NODES_GAUSS, warp=0.1)
    small_mesh, small_cfg, small_q = cases.tgv_case(n=2, order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO,
                                                    perturbation=0.05, seed=11)
    assert big_mesh.ndof > 3 * 8192 > small_mesh.ndof  # several blocks of partials, then one
    for mesh, cfg, q, cfl, dcfl in ((big_mesh, big_cfg, big_q, 0.4, 0.4), (small_mesh, small_cfg, small_q, 0.5, 1e5)):
        with NavierStokesDG(mesh, cfg) as g:
            g.set_state(q)
            ref = g.max_time_step(cfl, dcfl)
        got = _noalloc_dt(mesh, cfg, q, torch, cfl, dcfl)
        assert abs(got - ref) <= TOL * ref, (got, ref)


def test_noalloc_max_dt_euler_case_on_a_side_stream():
    """The Euler path (no viscous limit) on a stream other than the default one, twice in a row."""
    torch = pytest.importorskip("torch")
    mesh, cfg, q = cases.vortex_case(n=5, order=4, nodes=_abi.DG_NODES_GAUSS)
    assert cfg.physics().navier_stokes == 0
    with NavierStokesDG(mesh, cfg) as g:
        g.set_state(q)
        ref = g.max_time_step(0.4, 0.4)
    side = torch.cuda.Stream()
    for _ in range(2):
        got = _noalloc_dt(mesh, cfg, q, torch, 0.4, 0.4, stream=side)
        assert abs(got - ref) <= TOL * ref, (got, ref)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = _abi.lib()
    limit = L.dg_max_dt_noalloc_max_dof()
    assert limit == 67108864
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = x.data_ptr()
    dt = C.c_double()
    phys = _abi.DgPhysics(0.1, 1600.0, 0.72, 1)
    rc = L.dg_max_dt_noalloc(p, p, p, p, p, limit + 1, 3, 0, C.byref(phys), 0.4, 0.4, None, C.byref(dt))
    assert rc == _abi.DG_ERR_INVALID
    assert b"static scratch" in L.dg_last_error()
