"""The tensor-core building blocks (tcgen05 TF32 MMAs accumulated in tensor memory) against numpy:
the canonical operand layout, the descriptors and the TMEM read-back of C = A B^T with A 128 x 8 and
B 16 x 8. A single TF32 product is accurate to about 2^-11 relative; the three-term split product
(a_hi b_hi + a_hi b_lo + a_lo b_hi) to about 2^-20, the accuracy the tensor-core contractions of the
volume kernel rely on."""
import ctypes as C

import numpy as np
import pytest

from horses3d_gb300 import _abi
from horses3d_gb300.mesh import nodal_storage

pytestmark = pytest.mark.gpu


def _run(a, b, split):
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    c = np.zeros((128, 16), dtype=np.float32)
    fp = C.POINTER(C.c_float)
    _abi.check(_abi.lib().dg_tc_selftest(a.ctypes.data_as(fp), b.ctypes.data_as(fp), c.ctypes.data_as(fp), split),
               "dg_tc_selftest")
    return c


def test_identity_picks_the_columns():
    """B = [I_8; 0]: every row of C repeats the row of A (exact for TF32-representable inputs), so
    a transposed or shifted operand layout shows up at once."""
    rng = np.random.default_rng(1)
    a = rng.integers(-64, 64, size=(128, 8)).astype(np.float32) / 8.0  # TF32-exact values
    b = np.zeros((16, 8), np.float32)
    b[:8, :8] = np.eye(8)
    c = _run(a, b, 0)
    assert np.array_equal(c[:, :8], a) and np.all(c[:, 8:] == 0)


@pytest.mark.parametrize("split,tol", [(0, 2.0 ** -10), (1, 2.0 ** -19)])
def test_derivative_matrix_product(split, tol):
    """The N = 5 Gauss derivative matrix padded to K = 8 (and two end-value rows) applied to random
    lines: the error relative to sum |a||b| of each entry."""
    rng = np.random.default_rng(2)
    a = np.zeros((128, 8), np.float32)
    a[:, :6] = rng.uniform(-1, 1, size=(128, 6))
    _, _, d = nodal_storage(_abi.DG_NODES_GAUSS, 5)
    b = np.zeros((16, 8), np.float32)
    b[:6, :6] = np.asarray(d).reshape(6, 6)
    b[6, :6] = rng.uniform(-1, 1, 6)
    b[7, :6] = rng.uniform(-1, 1, 6)
    c = _run(a, b, split)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    scale = np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64).T + 1e-30
    err = np.max(np.abs(c - ref) / scale)
    assert err <= tol, err


# ---- the tensor-core form of the volume kernel (DG_PRECISION_MIXED_TC) ----
def _tgv_n5(precision, n=4):
    import cases

    return cases.tgv_case(n=n, order=5, nodes=_abi.DG_NODES_GAUSS, riemann=_abi.DG_RIEMANN_LXF, warp=0.1,
                          perturbation=0.01, seed=3, precision=precision)


def test_tensor_core_form_matches_the_oracle_and_the_fp32_form():
    """Curvilinear Taylor-Green, N = 5 Gauss, LxF, BR1: ten RK3 steps of the tensor-core form stay
    within 1e-6 relative L2 of the FP64 oracle (the mixed form's bar), and the lifted gradient of one
    right-hand side within 1e-5 of the oracle's."""
    import oracle
    from horses3d_gb300.problems import rel_l2
    from horses3d_gb300.solver import NavierStokesDG

    mesh, cfg, q0 = _tgv_n5(_abi.DG_PRECISION_MIXED_TC)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    o.rhs(0.0)
    with NavierStokesDG(mesh, cfg) as g:
        g.set_state(q0)
        g.compute_time_derivative(0.0)
        for f in (_abi.DG_FIELD_UX, _abi.DG_FIELD_UY, _abi.DG_FIELD_UZ):
            ref = o.get(f)
            err = np.max(np.abs(g.get(f) - ref)) / np.max(np.abs(ref))
            assert err <= 1e-5, (f, err)
        dt = 2e-3
        for s in range(10):
            o.rk3_step(s * dt, dt)
        g.set_state(q0)
        g.run_steps(10, 0.0, dt=dt)
        w = mesh.quadrature_weights()
        err = rel_l2(g.Q, o.get(0), w)
        assert np.all(err <= 1e-6), err


def test_tensor_core_form_rejects_other_configurations():
    import cases
    from horses3d_gb300.solver import NavierStokesDG

    for mesh, cfg, _ in (cases.tgv_case(n=2, order=3, nodes=_abi.DG_NODES_GAUSS, precision=_abi.DG_PRECISION_MIXED_TC),
                         cases.tgv_case(n=2, order=5, nodes=_abi.DG_NODES_GAUSS_LOBATTO,
                                        precision=_abi.DG_PRECISION_MIXED_TC)):
        with pytest.raises(_abi.DgError, match="tensor-core form"):
            NavierStokesDG(mesh, cfg)
