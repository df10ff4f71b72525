"""Host-side hexahedral mesh (the HexMesh of the reference) built by the native library.

``HexMesh.from_specmesh`` reads a SpecMesh file (Read_SpecMesh.f90:36-342); ``HexMesh.box`` builds
the periodic boxes of the benchmark cases directly. Both run the same connectivity and FP64
geometry code (HexMesh.f90:356-736, 2677-2990; MappedGeometry.f90:64-760) and expose the arrays as
numpy views in the reference's layouts.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi


class HexMesh:
    def __init__(self, handle: C.c_void_p):
        self._h = handle
        self.desc = _abi.DgMeshDesc()
        _abi.check(_abi.lib().h3d_mesh_describe(self._h, C.byref(self.desc)), "h3d_mesh_describe")
        d = self.desc
        self.n_elements = int(d.n_elements)
        self.node_type = int(d.node_type)
        self.order = np.ctypeslib.as_array(d.order, shape=(self.n_elements, 3)).copy()
        p = self.order + 1
        self.nodes_per_element = np.prod(p, axis=1)
        self.elem_offset = np.concatenate([[0], np.cumsum(self.nodes_per_element)]).astype(np.int64)
        self.ndof = int(self.elem_offset[-1])
        self.n_faces = int(d.n_faces)
        nf = np.ctypeslib.as_array(d.face_nf, shape=(self.n_faces, 2)) if self.n_faces else np.zeros((0, 2), np.int32)
        self.face_points = int(np.sum((nf[:, 0] + 1) * (nf[:, 1] + 1)))
        L = _abi.lib()
        self.zone_names = [L.h3d_mesh_zone_name(self._h, z).decode() for z in range(L.h3d_mesh_zone_count(self._h))]
        self.n_boundary_faces = 0
        if d.face_boundary:
            fb = np.ctypeslib.as_array(d.face_boundary, shape=(self.n_faces,))
            self.n_boundary_faces = int(np.count_nonzero(fb >= 0))

    def with_boundaries(self, table) -> _abi.DgMeshDesc:
        """A copy of the mesh description whose `boundaries` points at `table` (one DgBoundary per
        zone, in zone_names order). The caller keeps `table` alive while the description is used."""
        if len(table) != len(self.zone_names):
            raise ValueError(f"{len(table)} boundary conditions for {len(self.zone_names)} zones")
        d = _abi.DgMeshDesc()
        C.pointer(d)[0] = self.desc
        d.n_boundaries = len(table)
        d.boundaries = C.cast(table, C.POINTER(_abi.DgBoundary)) if len(table) else None
        return d

    # -- construction -------------------------------------------------------------------------
    @classmethod
    def from_specmesh(cls, path: str, order, node_type: int = _abi.DG_NODES_GAUSS,
                      periodic: str = "front:back,bottom:top,left:right") -> "HexMesh":
        h = C.c_void_p()
        if np.ndim(order) == 1 and len(order) == 3:  # one (Nx, Ny, Nz) for every element
            with open(path) as fh:
                n_elements = int(fh.readline().split()[1])  # header: nodes, elements, boundary order
            order = np.tile(np.asarray(order, dtype=np.int32), (n_elements, 1))
        if np.ndim(order) == 0:
            rc = _abi.lib().h3d_mesh_read_specmesh(str(path).encode(), node_type, int(order), None,
                                                   periodic.encode(), C.byref(h))
        else:
            o = np.ascontiguousarray(order, dtype=np.int32).reshape(-1)
            rc = _abi.lib().h3d_mesh_read_specmesh(str(path).encode(), node_type, 0, _abi.i32ptr(o),
                                                   periodic.encode(), C.byref(h))
        _abi.check(rc, "h3d_mesh_read_specmesh")
        return cls(h)

    @classmethod
    def box(cls, n, lo, hi, order, node_type: int = _abi.DG_NODES_GAUSS, warp: float = 0.0,
            patch_order: int = 0, periodic: str | None = None) -> "HexMesh":
        """Box of n^3 (or nx*ny*nz) hexahedra. periodic: the periodic zone pairs over left/right (x),
        front/back (y), bottom/top (z); None makes all three directions periodic, the zones left out
        are boundary zones."""
        nx, ny, nz = (n, n, n) if np.ndim(n) == 0 else n
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        h = C.c_void_p()
        spec = "front:back,bottom:top,left:right" if periodic is None else periodic
        if np.ndim(order) == 0:
            uniform, optr = int(order), None
        else:
            o = np.ascontiguousarray(order, dtype=np.int32).reshape(-1)
            uniform, optr = 0, _abi.i32ptr(o)
        rc = _abi.lib().h3d_mesh_box_zones(nx, ny, nz, _abi.f64ptr(lo), _abi.f64ptr(hi), float(warp), int(patch_order),
                                           node_type, uniform, optr, spec.encode(), C.byref(h))
        _abi.check(rc, "h3d_mesh_box")
        return cls(h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _abi.lib().h3d_mesh_free(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = None

    # -- array views ----------------------------------------------------------------------------
    def _view(self, ptr, n):
        return np.ctypeslib.as_array(ptr, shape=(n,))

    @property
    def x(self):
        return self._view(self.desc.x, 3 * self.ndof).reshape(self.ndof, 3)

    @property
    def jacobian(self):
        return self._view(self.desc.jacobian, self.ndof)

    @property
    def volume(self) -> float:
        return float(_abi.lib().h3d_mesh_volume(self._h))

    def quadrature_weights(self) -> np.ndarray:
        """w_i w_j w_k J at every node, element by element (the volume quadrature of
        MappedGeometry.f90:132-135), for any per-element orders."""
        out = np.empty(self.ndof)
        J = self.jacobian
        local = np.concatenate([np.arange(n) for n in self.nodes_per_element]) if self.n_elements else np.zeros(0, int)
        for key in {tuple(int(v) for v in o) for o in self.order}:
            ws = [nodal_storage(self.node_type, n)[1] for n in key]
            w3 = (ws[2][:, None, None] * ws[1][None, :, None] * ws[0][None, None, :]).reshape(-1)
            for e in np.nonzero(np.all(self.order == key, axis=1))[0]:
                s, t = self.elem_offset[e], self.elem_offset[e + 1]
                out[s:t] = w3[local[s:t]] * J[s:t]
        return out

    def uniform_order(self):
        """(N, N, N) when every element has the same isotropic order, else None."""
        o = self.order
        if np.all(o == o[0, 0]):
            return int(o[0, 0])
        return None


def nodal_storage(node_type: int, n: int):
    x = np.zeros(n + 1)
    w = np.zeros(n + 1)
    d = np.zeros((n + 1) * (n + 1))
    _abi.check(_abi.lib().h3d_nodal_storage(node_type, n, _abi.f64ptr(x), _abi.f64ptr(w), _abi.f64ptr(d)),
               "h3d_nodal_storage")
    return x, w, d.reshape(n + 1, n + 1)
