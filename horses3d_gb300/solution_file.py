"""HORSES3D solution files (.hsol; io/SolutionFile.f90, HexMesh_SaveSolution/LoadSolution in
HexMesh.f90) through the native reader and writer: read the header, read Q (and the gradients of a
type-3 file) for given element orders, write type-2 or type-3 files."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi

SOLUTION_FILE = 2
SOLUTION_AND_GRADIENTS_FILE = 3


def read_header(path) -> _abi.SolutionHeader:
    h = _abi.SolutionHeader()
    _abi.check(_abi.lib().h3d_read_solution_header(str(path).encode(), C.byref(h)), "h3d_read_solution_header")
    return h


def read(path, orders, gradients: bool = False):
    """Q (5 per node, element after element) and, if asked, the gradients U_x, U_y, U_z per element."""
    orders = np.ascontiguousarray(orders, dtype=np.int32).reshape(-1, 3)
    nodes = int(np.sum(np.prod(orders + 1, axis=1)))
    q = np.empty(5 * nodes)
    g = np.empty(15 * nodes) if gradients else None
    _abi.check(_abi.lib().h3d_read_solution(str(path).encode(), orders.shape[0], _abi.i32ptr(orders.reshape(-1)),
                                            _abi.f64ptr(q), _abi.f64ptr(g) if g is not None else None),
               "h3d_read_solution")
    return (q, g) if gradients else q


def write(path, header: _abi.SolutionHeader, orders, q, gradients=None) -> None:
    orders = np.ascontiguousarray(orders, dtype=np.int32).reshape(-1)
    q = np.ascontiguousarray(q, dtype=np.float64)
    g = None if gradients is None else np.ascontiguousarray(gradients, dtype=np.float64)
    _abi.check(_abi.lib().h3d_write_solution(str(path).encode(), C.byref(header), _abi.i32ptr(orders), _abi.f64ptr(q),
                                             _abi.f64ptr(g) if g is not None else None), "h3d_write_solution")
