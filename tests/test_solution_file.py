"""HORSES3D solution files (.hsol): the native reader and writer against files the reference itself
wrote (read when the reference tree is mounted): a NavierStokes restart file (type 2, 1,600 N=3
elements) and a file with gradients (type 3). Reading and writing back gives the same bytes."""
from pathlib import Path

import numpy as np
import pytest

from horses3d_gb300 import _abi, solution_file

REF = Path("/root/reference/Solver/test")
RESTART = REF / "NavierStokes" / "DualTimeStepping" / "RESULTS" / "Restart.hsol"
WITH_GRADIENTS = REF / "AddOns" / "horsesConverter" / "Files" / "Nodes_3.hsol"


@pytest.mark.skipif(not RESTART.exists(), reason="reference tree not mounted")
def test_reference_restart_file_round_trips_byte_for_byte(tmp_path):
    h = solution_file.read_header(RESTART)
    assert (h.file_type, h.node_type, h.n_elements, h.iteration) == (2, 1, 1600, 1)
    assert h.time == pytest.approx(0.01) and list(h.refs)[0] == 1.4 and list(h.refs)[5] == pytest.approx(0.3)
    orders = np.full((1600, 3), 3, dtype=np.int32)
    q = solution_file.read(RESTART, orders)
    rho = q.reshape(-1, 5)[:, 0]
    assert q.size == 5 * 1600 * 64 and np.all(rho > 0) and np.all(np.isfinite(q))
    out = tmp_path / "copy.hsol"
    solution_file.write(out, h, orders, q)
    assert out.read_bytes() == RESTART.read_bytes()


@pytest.mark.skipif(not WITH_GRADIENTS.exists(), reason="reference tree not mounted")
def test_reference_file_with_gradients_round_trips(tmp_path):
    h = solution_file.read_header(WITH_GRADIENTS)
    assert (h.file_type, h.n_elements) == (3, 3)
    orders = np.full((3, 3), 1, dtype=np.int32)
    q, g = solution_file.read(WITH_GRADIENTS, orders, gradients=True)
    out = tmp_path / "copy.hsol"
    solution_file.write(out, h, orders, q, g)
    assert out.read_bytes() == WITH_GRADIENTS.read_bytes()


def test_writer_reader_and_errors(tmp_path):
    rng = np.random.default_rng(1)
    orders = np.array([[1, 2, 3], [3, 3, 3], [2, 1, 1]], dtype=np.int32)
    nodes = int(np.sum(np.prod(orders + 1, axis=1)))
    q = rng.standard_normal(5 * nodes)
    h = _abi.SolutionHeader()
    h.name = b"RESULTS/test.hsol"
    h.file_type, h.node_type, h.n_elements, h.iteration, h.time = 2, 2, 3, 7, 0.25
    p = tmp_path / "t.hsol"
    solution_file.write(p, h, orders, q)
    assert p.stat().st_size == 204 + 3 * 20 + 8 * 5 * nodes + 4
    assert np.array_equal(solution_file.read(p, orders), q)
    with pytest.raises(_abi.DgError):  # orders that do not match the records
        solution_file.read(p, np.full((3, 3), 2, dtype=np.int32))
    with pytest.raises(_abi.DgError):  # no gradients in a type-2 file
        solution_file.read(p, orders, gradients=True)
    p.write_bytes(p.read_bytes()[:300])
    with pytest.raises(_abi.DgError):
        solution_file.read(p, orders)
