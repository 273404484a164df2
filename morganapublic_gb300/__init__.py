"""GB300 (sm_103a) finite-element operator path of morganaPublic.

Python mirror of the reference's builder interface over the C ABI of
libmorgana_gpu.so (include/morgana_gpu.h):

    reference (C++ templates)                       here
    ---------------------------------------------   -----------------------------------
    meshInit3d::gmMesh_to_stdB + dofMapStatic3d      Mesh(xyz, conn, order, edge_rule)
                                                     Mesh.load_gmsh(path, order, edge_rule)
    matrixBuilder<localMatrixEL3d<...>>(op)          MatrixBuilder(mesh)
      .buildEpetraCrs(matrix)                          .build_crs(op, coeff, c, quad, prec)
    vectorBuilder<localVectorEL3d<...>>              MatrixBuilder.build_vector(field, scale, quad)
      .buildEpetraVector(vector)
    Epetra_Operator::Apply                           MatrixBuilder.apply(values, x)
    belosBlockCG::solve                              MatrixBuilder.cg(values, b, ...)

Device memory is held in torch tensors (torch is used for allocation and
streams only); every computation runs in the CUDA library.  There is no CPU
fallback: the compute calls raise when the library or the GPU is missing.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import meshgen  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libmorgana_gpu.so")

MG_OK, MG_ERR_INVALID_ARG, MG_ERR_CUDA, MG_ERR_ALLOC, MG_ERR_BAD_MESH = 0, 1, 2, 3, 4
MG_ERR_NOT_CONVERGED, MG_ERR_UNSUPPORTED, MG_ERR_IO, MG_ERR_SIZE = 5, 6, 7, 8
EDGES = {"lex": 0, "first": 1}
OPS = {"stiff_kappa": 0, "stiff_const": 1, "mass": 2, "mass_coeff": 3}
PRECS = {"f64": 0, "f32": 1, "f64_native": 2}  # f64_native: assembly in native FP64 (full range)
PRECOND = {None: 0, "none": 0, "jacobi": 1}


class MorganaError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: {message} (status {status})")
        self.status = status


class _MeshInfo(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int64), ("n_elements", ctypes.c_int64), ("n_edges", ctypes.c_int64),
                ("ndof", ctypes.c_int64), ("order", ctypes.c_int32), ("edge_rule", ctypes.c_int32),
                ("min_det", ctypes.c_double)]


class CgInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("outer_iterations", ctypes.c_int32),
                ("converged", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("rel_residual", ctypes.c_double), ("seconds", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class SlotMapInfo(ctypes.Structure):
    _fields_ = [("n_upper", ctypes.c_int64), ("n_groups", ctypes.c_int64), ("n_diag", ctypes.c_int64),
                ("n_contrib", ctypes.c_int64), ("n_src", ctypes.c_int64), ("n_elem", ctypes.c_int64),
                ("nunique", ctypes.c_int32), ("elem_major", ctypes.c_int32), ("rows_per_block", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class BlockMapInfo(ctypes.Structure):
    _fields_ = [("n_upper", ctypes.c_int64), ("n_contrib", ctypes.c_int64), ("n_blocks", ctypes.c_int64),
                ("n_groups", ctypes.c_int64), ("n_src", ctypes.c_int64), ("n_runs", ctypes.c_int64),
                ("n_shared", ctypes.c_int64), ("n_shared_groups", ctypes.c_int64), ("n_partial", ctypes.c_int64),
                ("n_elem", ctypes.c_int64), ("nunique", ctypes.c_int32), ("elems_per_block", ctypes.c_int32)]


_P = ctypes.c_void_p
_I32, _I64, _D = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
# name -> argtypes; every function returns mg_status (int) unless listed in _RESTYPES
class LagrangeInfo(ctypes.Structure):
    _fields_ = [("n_faces", _I64), ("n_multipliers", _I64), ("ndof", _I64), ("nnz_b", _I64),
                ("nnz_saddle", _I64), ("nnz_mtm", _I64), ("n_mtm_products", _I64), ("n_edge_multipliers", _I64),
                ("nnz_mmt", _I64), ("n_mmt_products", _I64)]


class SaddleScales(ctypes.Structure):
    _fields_ = [("eye_field", ctypes.c_double), ("eye_lam", ctypes.c_double), ("mtm", ctypes.c_double),
                ("mmt", ctypes.c_double)]


SIGNATURES = {
    "mg_mesh_create": [ctypes.POINTER(_P), _I64, _P, _I64, _P, _I32, _I32],
    "mg_mesh_create_device": [ctypes.POINTER(_P), _I64, _P, _I64, _P, _I32, _I32, _P],
    "mg_mesh_load_gmsh": [ctypes.POINTER(_P), ctypes.c_char_p, _I32, _I32],
    "mg_mesh_destroy": [_P],
    "mg_mesh_get_info": [_P, ctypes.POINTER(_MeshInfo)],
    "mg_mesh_export_dofs": [_P, _P],
    "mg_mesh_export_edges": [_P, _P, _P],
    "mg_mesh_export_geometry": [_P, _P, _P],
    "mg_mesh_export_triangles": [_P, ctypes.POINTER(_I64), _P, _P],
    "mg_pattern_build": [_P, ctypes.POINTER(_P)],
    "mg_pattern_build_device": [_P, ctypes.POINTER(_P), _P],
    "mg_plan_destroy": [_P],
    "mg_pattern_info": [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)],
    "mg_pattern_export": [_P, _P, _P],
    "mg_pattern_device": [_P, ctypes.POINTER(_P), ctypes.POINTER(_P)],
    "mg_plan_slot_map_info": [_P, ctypes.POINTER(SlotMapInfo)],
    "mg_plan_export_slot_map": [_P, _P, _P, _P, _P, _P],
    "mg_plan_block_map_info": [_P, ctypes.POINTER(BlockMapInfo)],
    "mg_plan_export_block_map": [_P, _P, _P, _P, _P, _P, _P, _P],
    "mg_plan_export_elem_order": [_P, _P],
    "mg_assemble": [_P, _I32, _P, _D, _I32, _I32, _P, _P],
    "mg_assemble_host": [_P, _I32, _P, _D, _I32, _I32, _P, _P],
    "mg_plan_status": [_P],
    "mg_assemble_rhs": [_P, _P, _P, _I32, _P, _P],
    "mg_apply_dirichlet": [_P, _P, _I32, _P, _P, _P],
    "mg_spmv": [_P, _I32, _P, _P, _P, _P],
    "mg_cg_solve": [_P, _P, _P, _P, _D, _I32, _I32, ctypes.POINTER(CgInfo), _P],
    "mg_cg_refined": [_P, _P, _P, _P, _P, _D, _I32, _I32, _D, _I32, ctypes.POINTER(CgInfo), _P],
    "mg_cg_solve_noalloc": [_P, _P, _P, _P, _D, _I32, _I32, ctypes.POINTER(CgInfo), _P],
    "mg_adjoint_grad": [_P, _P, _P, _I32, _P, _P],
    "mg_lagrange_build": [_P, _I32, _I64, _P, _I32, ctypes.POINTER(_P)],
    "mg_lagrange_destroy": [_P],
    "mg_lagrange_get_info": [_P, ctypes.POINTER(LagrangeInfo)],
    "mg_lagrange_export": [_P, _P, _P, _P],
    "mg_lagrange_pattern": [_P, _P, _P, _P, _P],
    "mg_lagrange_export_maps": [_P, _P, _P, _P],
    "mg_lagrange_assemble": [_P, _I32, _P, _P],
    "mg_lagrange_assemble_host": [_P, _I32, _P],
    "mg_saddle_assemble": [_P, _P, _P, ctypes.POINTER(SaddleScales), _P, _P],
    "mg_lagrange_export_products": [_P, _I32, _P, _P, _P],
    "mg_lagrange_export_edges": [_P, _P],
    "mg_saddle_spmv": [_P, _P, _P, _P, _P],
    "mg_lagrange_apply": [_P, _P, _P, _P, _P],
    "mg_status_string": [_I32],
    "mg_last_error": [],
    "mg_version": [],
}
_RESTYPES = {"mg_status_string": ctypes.c_char_p, "mg_last_error": ctypes.c_char_p, "mg_version": ctypes.c_char_p}

_lib = None


def lib():
    """Loads libmorgana_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m morganapublic_gb300.build` "
                              "(or __graft_entry__.build()) first")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = L
    return _lib


def _check(status: int, where: str):
    if status != MG_OK:
        raise MorganaError(status, where, lib().mg_last_error().decode())


def _ptr(a) -> int | None:
    """Raw pointer of a numpy array or a torch tensor (None passes through)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


def _stream_ptr(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("morganapublic_gb300 compute calls need a CUDA device; none is visible")
    return torch


class Mesh:
    """Tetrahedral mesh with its P1/P2 dof map (mg_mesh)."""

    def __init__(self, xyz, conn, order: int = 1, edge_rule: str = "lex", _handle=None,
                 edges_on_device: bool = False, stream=None):
        """edges_on_device: enumerate the P2 edges on the GPU (mg_mesh_create_device); identical result."""
        L = lib()
        h = _P()
        if _handle is None:
            xyz = np.ascontiguousarray(xyz, dtype=np.float64)
            conn = np.ascontiguousarray(conn, dtype=np.int32)
            if edges_on_device:
                _torch()
                _check(L.mg_mesh_create_device(ctypes.byref(h), xyz.shape[0], _ptr(xyz), conn.shape[0],
                                               _ptr(conn), order, EDGES[edge_rule], _stream_ptr(stream)),
                       "mg_mesh_create_device")
            else:
                _check(L.mg_mesh_create(ctypes.byref(h), xyz.shape[0], _ptr(xyz), conn.shape[0], _ptr(conn),
                                        order, EDGES[edge_rule]), "mg_mesh_create")
        else:
            h = _handle
        self._h = h
        info = _MeshInfo()
        _check(L.mg_mesh_get_info(self._h, ctypes.byref(info)), "mg_mesh_get_info")
        self.n_nodes, self.n_elements, self.ndof = info.n_nodes, info.n_elements, info.ndof
        self.order, self.min_det = info.order, info.min_det
        self.nb = 4 if order == 1 else 10

    @classmethod
    def load_gmsh(cls, path: str, order: int = 1, edge_rule: str = "lex") -> "Mesh":
        h = _P()
        _check(lib().mg_mesh_load_gmsh(ctypes.byref(h), path.encode(), order, EDGES[edge_rule]),
               "mg_mesh_load_gmsh")
        return cls(None, None, order, edge_rule, _handle=h)

    @property
    def n_edges(self) -> int:
        info = _MeshInfo()
        _check(lib().mg_mesh_get_info(self._h, ctypes.byref(info)), "mg_mesh_get_info")
        return info.n_edges

    def elem_dofs(self) -> np.ndarray:
        out = np.empty((self.n_elements, self.nb), dtype=np.int32)
        _check(lib().mg_mesh_export_dofs(self._h, _ptr(out)), "mg_mesh_export_dofs")
        return out

    def edges(self):
        """(edge_nodes (nE, 2), elem_edges (E, 6))"""
        L = lib()
        _check(L.mg_mesh_export_edges(self._h, None, None), "mg_mesh_export_edges")
        ne = self.n_edges
        en = np.empty((ne, 2), dtype=np.int32)
        ee = np.empty((self.n_elements, 6), dtype=np.int32)
        _check(L.mg_mesh_export_edges(self._h, _ptr(en), _ptr(ee)), "mg_mesh_export_edges")
        return en, ee

    def geometry(self):
        xyz = np.empty((self.n_nodes, 3), dtype=np.float64)
        conn = np.empty((self.n_elements, 4), dtype=np.int32)
        _check(lib().mg_mesh_export_geometry(self._h, _ptr(xyz), _ptr(conn)), "mg_mesh_export_geometry")
        return xyz, conn

    def triangles(self, geo_ids=None):
        """The Gmsh file's triangles (k, 3), file order, and their geoIds; with
        geo_ids, only the triangles of those geoIds (the test field's filter)."""
        n = _I64()
        _check(lib().mg_mesh_export_triangles(self._h, ctypes.byref(n), None, None), "mg_mesh_export_triangles")
        tris = np.empty((n.value, 3), dtype=np.int32)
        geo = np.empty(n.value, dtype=np.int32)
        _check(lib().mg_mesh_export_triangles(self._h, ctypes.byref(n), _ptr(tris), _ptr(geo)),
               "mg_mesh_export_triangles")
        if geo_ids is not None:
            keep = np.isin(geo, np.asarray(list(geo_ids)))
            tris, geo = tris[keep], geo[keep]
        return tris, geo

    def close(self):
        if getattr(self, "_h", None):
            lib().mg_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Csr:
    rowptr: np.ndarray
    colind: np.ndarray
    values: np.ndarray


class MatrixBuilder:
    """CSR pattern + GPU assembly plan of a mesh (mg_plan); the counterpart of
    the reference's matrixBuilder / vectorBuilder and of the operator Belos uses."""

    def __init__(self, mesh: Mesh, pattern_on_device: bool = False, stream=None):
        """pattern_on_device: build the CSR pattern, the element order and the slot map on
        the GPU (mg_pattern_build_device) instead of the host; the arrays are identical."""
        self.mesh = mesh
        h = _P()
        if pattern_on_device:
            _torch()
            _check(lib().mg_pattern_build_device(mesh._h, ctypes.byref(h), _stream_ptr(stream)),
                   "mg_pattern_build_device")
        else:
            _check(lib().mg_pattern_build(mesh._h, ctypes.byref(h)), "mg_pattern_build")
        self._h = h
        nd, nz = _I64(), _I64()
        _check(lib().mg_pattern_info(h, ctypes.byref(nd), ctypes.byref(nz)), "mg_pattern_info")
        self.ndof, self.nnz = nd.value, nz.value

    # ----------------------------------------------------------- pattern --
    def pattern(self):
        rp = np.empty(self.ndof + 1, dtype=np.int32)
        ci = np.empty(self.nnz, dtype=np.int32)
        _check(lib().mg_pattern_export(self._h, _ptr(rp), _ptr(ci)), "mg_pattern_export")
        return rp, ci

    def elem_order(self) -> np.ndarray:
        """The assembly's element order (a Morton curve of the centroids): element ids."""
        out = np.empty(self.mesh.n_elements, dtype=np.int32)
        _check(lib().mg_plan_export_elem_order(self._h, _ptr(out)), "mg_plan_export_elem_order")
        return out

    def block_map_info(self) -> BlockMapInfo:
        """Sizes of the one-pass P1 assembly's block map (mg_plan_block_map_info)."""
        info = BlockMapInfo()
        _check(lib().mg_plan_block_map_info(self._h, ctypes.byref(info)), "mg_plan_block_map_info")
        return info

    def export_block_map(self) -> dict:
        """The P1 assembly's block map (mg_plan_export_block_map); makes the plan device-resident."""
        info = self.block_map_info()
        out = {"elem_order": np.empty(info.n_elem, dtype=np.int32),
               "bgrp": np.empty(info.n_blocks + 1, dtype=np.int32),
               "goff": np.empty(info.n_groups + 1, dtype=np.int32),
               "src": np.empty(info.n_src, dtype=np.uint16),
               "out": np.empty((32 * info.n_groups, 2), dtype=np.int32),
               "sgoff": np.empty(info.n_shared_groups + 1, dtype=np.int32),
               "sout": np.empty((32 * info.n_shared_groups, 2), dtype=np.int32)}
        _check(lib().mg_plan_export_block_map(self._h, *[_ptr(out[k]) for k in
                                                         ("elem_order", "bgrp", "goff", "src", "out", "sgoff",
                                                          "sout")]),
               "mg_plan_export_block_map")
        out["info"] = info
        return out

    def slot_map_info(self) -> SlotMapInfo:
        info = SlotMapInfo()
        _check(lib().mg_plan_slot_map_info(self._h, ctypes.byref(info)), "mg_plan_slot_map_info")
        return info

    def export_slot_map(self) -> dict:
        """The assembly's slot map (mg_plan_export_slot_map); makes the plan device-resident."""
        info = self.slot_map_info()
        out = {"elem_order": np.empty(info.n_elem, dtype=np.int32),
               "goff": np.empty(info.n_groups + 1, dtype=np.int32),
               "uslot": np.empty(info.n_upper, dtype=np.int32),
               "umirror": np.empty(info.n_upper, dtype=np.int32),
               "src": np.empty(info.n_src, dtype=np.uint32)}
        _check(lib().mg_plan_export_slot_map(self._h, *[_ptr(out[k]) for k in
                                                        ("elem_order", "goff", "uslot", "umirror", "src")]),
               "mg_plan_export_slot_map")
        out["info"] = info
        return out

    def device_pattern(self):
        """(rowptr, colind) as int32 torch tensors on the GPU (copies)."""
        torch = _torch()
        rp, ci = _P(), _P()
        _check(lib().mg_pattern_device(self._h, ctypes.byref(rp), ctypes.byref(ci)), "mg_pattern_device")
        rph, cih = self.pattern()
        return torch.from_numpy(rph).cuda(), torch.from_numpy(cih).cuda()

    # ---------------------------------------------------------- assembly --
    def assemble(self, op: str = "stiff_kappa", coeff=None, c: float = 1.0, quad: int = 4, prec: str = "f64",
                 out=None, stream=None):
        """CSR values on the GPU (torch tensor of nnz float64/float32)."""
        torch = _torch()
        dt = torch.float32 if prec == "f32" else torch.float64
        if out is None:
            out = torch.empty(self.nnz, dtype=dt, device="cuda")
        if coeff is not None:
            coeff = torch.as_tensor(coeff, dtype=torch.float64, device="cuda").contiguous()
        _check(lib().mg_assemble(self._h, OPS[op], _ptr(coeff), float(c), quad, PRECS[prec], _ptr(out),
                                 _stream_ptr(stream)), "mg_assemble")
        return out

    def build_crs(self, op: str = "stiff_kappa", coeff=None, c: float = 1.0, quad: int = 4,
                  prec: str = "f64") -> Csr:
        """Host-buffer assembly (what buildEpetraCrs hands to Epetra): pattern + values."""
        _torch()
        vals = np.empty(self.nnz, dtype=np.float32 if prec == "f32" else np.float64)
        cf = None if coeff is None else np.ascontiguousarray(coeff, dtype=np.float64)
        _check(lib().mg_assemble_host(self._h, OPS[op], _ptr(cf), float(c), quad, PRECS[prec], _ptr(vals),
                                      _stream_ptr(None)), "mg_assemble_host")
        rp, ci = self.pattern()
        return Csr(rp, ci, vals)

    def build_vector(self, field=None, elem_scale=None, quad: int = 4, out=None, stream=None):
        torch = _torch()
        if out is None:
            out = torch.empty(self.ndof, dtype=torch.float64, device="cuda")
        f = None if field is None else torch.as_tensor(field, dtype=torch.float64, device="cuda").contiguous()
        s = None if elem_scale is None else torch.as_tensor(elem_scale, dtype=torch.float64,
                                                            device="cuda").contiguous()
        _check(lib().mg_assemble_rhs(self._h, _ptr(f), _ptr(s), quad, _ptr(out), _stream_ptr(stream)),
               "mg_assemble_rhs")
        return out

    def status(self):
        """Synchronises and raises if an earlier asynchronous assembly recorded a device-side failure."""
        _check(lib().mg_plan_status(self._h), "mg_plan_status")

    def apply_dirichlet(self, values, mask, b=None, stream=None):
        torch = _torch()
        m = torch.as_tensor(mask, device="cuda").to(torch.uint8).contiguous()
        prec = "f64" if values.dtype == torch.float64 else "f32"
        _check(lib().mg_apply_dirichlet(self._h, _ptr(m), PRECS[prec], _ptr(values), _ptr(b),
                                        _stream_ptr(stream)), "mg_apply_dirichlet")
        return values

    # ------------------------------------------------------------- solve --
    def apply(self, values, x, out=None, stream=None):
        """y = A x (Epetra_Operator::Apply)."""
        torch = _torch()
        prec = "f64" if values.dtype == torch.float64 else "f32"
        if out is None:
            out = torch.empty(self.ndof, dtype=values.dtype, device="cuda")
        _check(lib().mg_spmv(self._h, PRECS[prec], _ptr(values), _ptr(x), _ptr(out), _stream_ptr(stream)),
               "mg_spmv")
        return out

    def cg(self, values, b, x0=None, rtol: float = 1e-10, maxit: int = 10000, precond="jacobi", stream=None,
           raise_on_fail: bool = True):
        torch = _torch()
        x = torch.zeros_like(b) if x0 is None else x0.clone()
        info = CgInfo()
        st = lib().mg_cg_solve(self._h, _ptr(values), _ptr(b), _ptr(x), rtol, maxit, PRECOND[precond],
                               ctypes.byref(info), _stream_ptr(stream))
        if raise_on_fail or st not in (MG_OK, MG_ERR_NOT_CONVERGED):
            _check(st, "mg_cg_solve")
        return x, info

    def cg_refined(self, values64, values32, b, x0=None, rtol: float = 1e-10, max_outer: int = 200,
                   max_inner: int = 100000, inner_rtol: float = 1e-2, precond="jacobi", stream=None,
                   raise_on_fail: bool = True):
        torch = _torch()
        x = torch.zeros_like(b) if x0 is None else x0.clone()
        info = CgInfo()
        st = lib().mg_cg_refined(self._h, _ptr(values64), _ptr(values32), _ptr(b), _ptr(x), rtol, max_outer,
                                 max_inner, inner_rtol, PRECOND[precond], ctypes.byref(info),
                                 _stream_ptr(stream))
        if raise_on_fail or st not in (MG_OK, MG_ERR_NOT_CONVERGED):
            _check(st, "mg_cg_refined")
        return x, info

    def adjoint_grad(self, u, lam, quad: int = 4, out=None, stream=None):
        torch = _torch()
        if out is None:
            out = torch.empty(self.mesh.n_elements, dtype=torch.float64, device="cuda")
        _check(lib().mg_adjoint_grad(self._h, _ptr(u), _ptr(lam), quad, _ptr(out), _stream_ptr(stream)),
               "mg_adjoint_grad")
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().mg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LagrangeBuilder:
    """Dirichlet data the reference way (mg_lagrange): P1 multipliers on the
    boundary triangles, B = opLA3dA (multiplier x field) and the saddle matrix
    [K B^T; B 0] of epetraSaddleAssembler.  Keeps a reference to its
    MatrixBuilder, whose plan must outlive it."""

    def __init__(self, builder: MatrixBuilder, tris=None, lam_diag: bool = False, test_order: int = 1,
                 mtm: bool = False, mmt: bool = False):
        """tris: (k, 3) node ids of the boundary triangles that carry multipliers
        (the test field's geoId filter); None = every boundary face.
        test_order: 1 = P1 multipliers (one per boundary node), 0 = P0 (one per
        triangle, in the order of tris), 2 = P2 (the P1 ones, then one per
        boundary edge in (min node, max node) order).  lam_diag: store the multiplier block's
        diagonal; mtm: merge B^T B into the field block (setMTM); mmt: merge
        B B^T into the multiplier block (setMMT)."""
        self.builder = builder
        self.test_order = test_order
        t = None if tris is None else np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
        flags = (1 if lam_diag else 0) | (2 if mtm else 0) | (4 if mmt else 0)
        h = _P()
        _check(lib().mg_lagrange_build(builder._h, int(test_order), 0 if t is None else t.shape[0], _ptr(t),
                                       flags, ctypes.byref(h)), "mg_lagrange_build")
        self._h = h
        info = LagrangeInfo()
        _check(lib().mg_lagrange_get_info(h, ctypes.byref(info)), "mg_lagrange_get_info")
        self.n_faces, self.n_multipliers = info.n_faces, info.n_multipliers
        self.ndof, self.nnz_b, self.nnz_saddle = info.ndof, info.nnz_b, info.nnz_saddle
        self.nnz_mtm, self.n_mtm_products = info.nnz_mtm, info.n_mtm_products
        self.n_edge_multipliers = info.n_edge_multipliers
        self.nnz_mmt, self.n_mmt_products = info.nnz_mmt, info.n_mmt_products

    def multipliers(self):
        """(node (P1) or face index (P0) of each multiplier, face element, face local index)."""
        lam = np.empty(self.n_multipliers, dtype=np.int32)
        fe = np.empty(self.n_faces, dtype=np.int32)
        fl = np.empty(self.n_faces, dtype=np.int32)
        _check(lib().mg_lagrange_export(self._h, _ptr(lam), _ptr(fe), _ptr(fl)), "mg_lagrange_export")
        return lam, fe, fl

    def pattern(self):
        """((B rowptr, colind), (saddle rowptr, colind))."""
        brp = np.empty(self.n_multipliers + 1, dtype=np.int32)
        bci = np.empty(self.nnz_b, dtype=np.int32)
        srp = np.empty(self.ndof + self.n_multipliers + 1, dtype=np.int32)
        sci = np.empty(self.nnz_saddle, dtype=np.int32)
        _check(lib().mg_lagrange_pattern(self._h, _ptr(brp), _ptr(bci), _ptr(srp), _ptr(sci)),
               "mg_lagrange_pattern")
        return (brp, bci), (srp, sci)

    def export_maps(self):
        """(b_src_ptr, b_src, s_src): the gather maps of the B and saddle kernels."""
        nb = 4 if self.builder.mesh.order == 1 else 10
        nt = {0: 1, 1: 3, 2: 6}[self.test_order]
        bp = np.empty(self.nnz_b + 1, dtype=np.int32)
        bs = np.empty(self.n_faces * nt * nb, dtype=np.int32)
        ss = np.empty(self.nnz_saddle, dtype=np.int32)
        _check(lib().mg_lagrange_export_maps(self._h, _ptr(bp), _ptr(bs), _ptr(ss)), "mg_lagrange_export_maps")
        return bp, bs, ss

    def assemble(self, quad: int = 1, out=None, stream=None):
        """Values of B (torch float64, nnz_b) with the face card quad (1, 3, 4, 6)."""
        torch = _torch()
        if out is not None:
            self._need(out, self.nnz_b, "out")
        if out is None:
            out = torch.empty(self.nnz_b, dtype=torch.float64, device="cuda")
        _check(lib().mg_lagrange_assemble(self._h, quad, _ptr(out), _stream_ptr(stream)), "mg_lagrange_assemble")
        return out

    @staticmethod
    def _need(t, n, what):
        torch = _torch()
        if t is None or not isinstance(t, torch.Tensor) or t.dtype != torch.float64 or not t.is_cuda \
                or t.numel() < n or not t.is_contiguous():
            raise ValueError(f"{what}: a contiguous float64 CUDA tensor of at least {n} entries is needed")

    def build_crs(self, quad: int = 1) -> Csr:
        """B with host buffers (what buildEpetraCrs hands to Epetra for localMatrixLA3d)."""
        _torch()
        vals = np.empty(self.nnz_b, dtype=np.float64)
        _check(lib().mg_lagrange_assemble_host(self._h, quad, _ptr(vals)), "mg_lagrange_assemble_host")
        (rp, ci), _ = self.pattern()
        return Csr(rp, ci, vals)

    def edge_multipliers(self):
        """P2: (min node, max node) of each edge multiplier (they follow the vertex ones)."""
        out = np.empty((self.n_edge_multipliers, 2), dtype=np.int32)
        _check(lib().mg_lagrange_export_edges(self._h, _ptr(out)), "mg_lagrange_export_edges")
        return out

    def export_products(self, which: str = "mtm"):
        """(pair_ptr, pairs (n, 2), slot) of the B^T B ("mtm") or B B^T ("mmt") block."""
        nnz, n = (self.nnz_mtm, self.n_mtm_products) if which == "mtm" else (self.nnz_mmt, self.n_mmt_products)
        pp = np.empty(nnz + 1, dtype=np.int32)
        pr = np.empty((n, 2), dtype=np.int32)
        sl = np.empty(nnz, dtype=np.int32)
        _check(lib().mg_lagrange_export_products(self._h, 2 if which == "mtm" else 4, _ptr(pp), _ptr(pr), _ptr(sl)),
               "mg_lagrange_export_products")
        return pp, pr, sl

    def saddle(self, k_values, b_values, eye_field: float = 0.0, eye_lam: float = 0.0, mtm_scale: float = 0.0,
               mmt_scale: float = 0.0, out=None, stream=None):
        """Values of [K + eye_field I + mtm_scale B^T B, B^T; B, eye_lam I + mmt_scale B B^T]
        (torch float64, nnz_saddle)."""
        torch = _torch()
        self._need(k_values, self.builder.nnz, "K values")
        if self.nnz_b:
            self._need(b_values, self.nnz_b, "B values")
        if out is not None:
            self._need(out, self.nnz_saddle, "out")
        if out is None:
            out = torch.empty(self.nnz_saddle, dtype=torch.float64, device="cuda")
        scales = SaddleScales(float(eye_field), float(eye_lam), float(mtm_scale), float(mmt_scale))
        _check(lib().mg_saddle_assemble(self._h, _ptr(k_values), _ptr(b_values), ctypes.byref(scales), _ptr(out),
                                        _stream_ptr(stream)), "mg_saddle_assemble")
        return out

    def saddle_apply(self, values, x, out=None, stream=None):
        torch = _torch()
        n = self.ndof + self.n_multipliers
        self._need(values, self.nnz_saddle, "saddle values")
        self._need(x, n, "x")
        if out is not None:
            self._need(out, n, "out")
        if out is None:
            out = torch.empty(self.ndof + self.n_multipliers, dtype=torch.float64, device="cuda")
        _check(lib().mg_saddle_spmv(self._h, _ptr(values), _ptr(x), _ptr(out), _stream_ptr(stream)),
               "mg_saddle_spmv")
        return out

    def apply(self, b_values, u, out=None, stream=None):
        """g = B u: the constraint right-hand side of nodal data u."""
        torch = _torch()
        if self.nnz_b:
            self._need(b_values, self.nnz_b, "B values")
        self._need(u, self.ndof, "u")
        if out is not None:
            self._need(out, self.n_multipliers, "out")
        if out is None:
            out = torch.empty(self.n_multipliers, dtype=torch.float64, device="cuda")
        _check(lib().mg_lagrange_apply(self._h, _ptr(b_values), _ptr(u), _ptr(out), _stream_ptr(stream)),
               "mg_lagrange_apply")
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().mg_lagrange_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def version() -> str:
    return lib().mg_version().decode()
