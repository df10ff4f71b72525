"""HORSES3D solution files (.hsol): the native reader and writer against files the reference itself
wrote (the small one is a committed fixture; the 4 MB restart file is read from the reference tree
named by $HORSES3D_REFERENCE, when set): a NavierStokes restart file (type 2, 1,600 N=3
elements) and a file with gradients (type 3). Reading and writing back gives the same bytes."""
from pathlib import Path

import numpy as np
import pytest

import cases
from horses3d_gb300 import _abi, solution_file

RESTART_REL = "Solver/test/NavierStokes/DualTimeStepping/RESULTS/Restart.hsol"
WITH_GRADIENTS_REL = "Solver/test/AddOns/horsesConverter/Files/Nodes_3.hsol"


def _reference_or_skip(rel, tmp_path):
    path = cases.reference_file(rel, tmp_path)
    if path is None:
        pytest.skip(f"{rel}: no fixture and no reference tree (set ${cases.REFERENCE_ENV})")
    return path


def test_reference_restart_file_round_trips_byte_for_byte(tmp_path):
    RESTART = _reference_or_skip(RESTART_REL, tmp_path)
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


def test_reference_file_with_gradients_round_trips(tmp_path):
    WITH_GRADIENTS = _reference_or_skip(WITH_GRADIENTS_REL, tmp_path)
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


def _write_sensor_file(path, file_type, orders, q, g=None, sensor=None):
    """A sensor solution file (type 9, or 10 with gradients) as HexMesh_SaveSolution writes it: each
    element record ends with the element's sensor value (HexMesh.f90:3522-3525)."""
    import struct

    out = bytearray(b"RESULTS/sensor.hsol".ljust(128))
    out += struct.pack("<4i", file_type, 1, len(orders), 3) + struct.pack("<d", 0.5) + struct.pack("<6d", *range(6))
    out += struct.pack("<i", 88)
    off = 0
    for e, o in enumerate(orders):
        np_ = int(np.prod(o + 1))
        out += struct.pack("<5i", 4, 5, *(o + 1))
        out += q[5 * off:5 * (off + np_)].tobytes()
        if g is not None:
            for d in range(3):
                out += g[15 * off + 5 * np_ * d:15 * off + 5 * np_ * (d + 1)].tobytes()
        out += struct.pack("<d", sensor[e])
        off += np_
    out += struct.pack("<i", 99)
    path.write_bytes(bytes(out))


def test_sensor_files_skip_the_sensor_value(tmp_path):
    """Types 9 and 10 carry one sensor value per element after its data (HexMesh.f90:4832 adds it to
    each record's position); Q and the gradients of every element read back exactly."""
    rng = np.random.default_rng(3)
    orders = np.array([[1, 2, 3], [3, 3, 3], [2, 1, 1], [2, 2, 2]], dtype=np.int32)
    nodes = int(np.sum(np.prod(orders + 1, axis=1)))
    q = rng.standard_normal(5 * nodes)
    g = rng.standard_normal(15 * nodes)
    sensor = rng.standard_normal(len(orders))
    p9, p10 = tmp_path / "s9.hsol", tmp_path / "s10.hsol"
    _write_sensor_file(p9, 9, orders, q, sensor=sensor)
    _write_sensor_file(p10, 10, orders, q, g, sensor=sensor)
    assert np.array_equal(solution_file.read(p9, orders), q)
    q10, g10 = solution_file.read(p10, orders, gradients=True)
    assert np.array_equal(q10, q) and np.array_equal(g10, g)
    with pytest.raises(_abi.DgError):  # no gradients in a type-9 file
        solution_file.read(p9, orders, gradients=True)


def test_non_solution_file_types_are_rejected(tmp_path):
    orders = np.full((2, 3), 1, dtype=np.int32)
    q = np.zeros(5 * 16)
    for file_type in (1, 4, 5, 6, 7, 8):
        p = tmp_path / f"t{file_type}.hsol"
        _write_sensor_file(p, 9, orders, q, sensor=np.zeros(2))
        b = bytearray(p.read_bytes())
        b[128:132] = np.int32(file_type).tobytes()
        p.write_bytes(bytes(b))
        with pytest.raises(_abi.DgError, match="not a solution file"):
            solution_file.read(p, orders)
