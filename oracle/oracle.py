"""ctypes front end of the CPU oracle (morgana_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker the parity tests, the smoke check and the
cpu_baseline leg of bench.py compare the CUDA path against.  The product
package never imports this module.

Each wrapper returns numpy arrays with 0-based indices; see morgana_oracle.c for
the reference file:line each function restates.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmorgana_oracle.so")

OPS = {"stiff_kappa": 0, "stiff_const": 1, "mass": 2, "mass_coeff": 3}
EDGES = {"lex": 0, "first": 1}
# quadrature names of the product (1, 4, 15, 64 points) -> reference card precision
QUAD_PREC = {1: 1, 4: 2, 15: 3, 64: 4}
# triangle cards of the boundary-face operator by point count -> reference precision
FACE_QUAD_PREC = {1: 1, 3: 2, 4: 3, 6: 4}
# local faces of linearTetra (geoShapes.cpp:681-688), 0-based
FACE_PTS = np.array([[0, 2, 1], [0, 1, 3], [1, 2, 3], [0, 3, 2]])

_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P, I64, I32, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        L.or_quad_rule.argtypes = [I32, P, P]
        L.or_local_matrix.argtypes = [I32, I32, I32, P, P, D, D, P]
        L.or_element_det.argtypes = [P, P]
        L.or_element_det.restype = D
        L.or_check_jacobian.argtypes = [I64, P, P, P, P]
        L.or_build_edges.argtypes = [I64, I64, P, I32, P, P, P]
        L.or_elem_dofs.argtypes = [I32, I64, I64, P, P, P]
        L.or_pattern.argtypes = [I32, I64, I64, P, P, P, I64, P]
        L.or_assemble_values.argtypes = [I32, I32, I32, P, I64, P, P, P, D, P, P, I64, P]
        L.or_assemble_rhs.argtypes = [I32, I32, P, I64, P, P, P, P, I64, P]
        L.or_apply_dirichlet.argtypes = [I64, P, P, P, P, P]
        L.or_spmv.argtypes = [I64, P, P, P, P, P]
        L.or_cg.argtypes = [I64, P, P, P, P, P, D, I32, I32, P, P]
        L.or_adjoint_grad.argtypes = [I32, I32, P, I64, P, P, P, P, P]
        L.or_basis_eval.argtypes = [I32, P, P]
        L.or_basis_grad.argtypes = [I32, P, P, P, P]
        L.or_tri_rule.argtypes = [I32, P, P]
        L.or_face_matrix.argtypes = [I32, I32, I32, P, P, I32, P]
        L.or_face_matrices.argtypes = [I32, I32, I32, P, I64, P, P, P, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def quad_rule(quad: int):
    Y = np.empty((64, 3))
    W = np.empty(64)
    n = lib().or_quad_rule(QUAD_PREC[quad], _p(Y), _p(W))
    return Y[:n].copy(), W[:n].copy()


def local_matrix(op, order, quad, xyz, nodes4, kappa=1.0, c=1.0):
    nb = 4 if order == 1 else 10
    mat = np.empty(nb * nb)
    nodes4 = np.ascontiguousarray(nodes4, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    rc = lib().or_local_matrix(OPS[op], order, QUAD_PREC[quad], _p(xyz), _p(nodes4), kappa, c, _p(mat))
    assert rc == 0
    return mat.reshape(nb, nb)  # [field i, test j]


def check_jacobian(xyz, conn):
    mn = ctypes.c_double()
    bad = ctypes.c_int64()
    rc = lib().or_check_jacobian(conn.shape[0], _p(xyz), _p(conn), ctypes.byref(mn), ctypes.byref(bad))
    return rc, mn.value, bad.value


def edges(n_nodes, conn, rule="lex"):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    E = conn.shape[0]
    ee = np.empty((E, 6), dtype=np.int32)
    en = np.empty((6 * E, 2), dtype=np.int32)
    ne = ctypes.c_int64()
    assert lib().or_build_edges(n_nodes, E, _p(conn), EDGES[rule], _p(ee), _p(en), ctypes.byref(ne)) == 0
    return en[: ne.value].copy(), ee


def elem_dofs(order, n_nodes, conn, elem_edge=None):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    nb = 4 if order == 1 else 10
    out = np.empty((conn.shape[0], nb), dtype=np.int32)
    ee = np.zeros((conn.shape[0], 6), dtype=np.int32) if elem_edge is None else np.ascontiguousarray(elem_edge)
    lib().or_elem_dofs(order, n_nodes, conn.shape[0], _p(conn), _p(ee), _p(out))
    return out


def pattern(order, ndof, dofs):
    nb = dofs.shape[1]
    cap = dofs.shape[0] * nb * nb + 1
    rp = np.empty(ndof + 1, dtype=np.int32)
    ci = np.empty(cap, dtype=np.int32)
    nnz = ctypes.c_int64()
    assert lib().or_pattern(order, ndof, dofs.shape[0], _p(dofs), _p(rp), _p(ci), cap, ctypes.byref(nnz)) == 0
    return rp, ci[: nnz.value].copy()


def assemble(op, order, quad, xyz, conn, dofs, rowptr, colind, coeff=None, c=1.0):
    vals = np.empty(colind.shape[0])
    cf = None if coeff is None else np.ascontiguousarray(coeff, dtype=np.float64)
    rc = lib().or_assemble_values(OPS[op], order, QUAD_PREC[quad], _p(xyz), conn.shape[0], _p(conn), _p(dofs),
                                  _p(cf), c, _p(rowptr), _p(colind), rowptr.shape[0] - 1, _p(vals))
    assert rc == 0
    return vals


def assemble_rhs(order, quad, xyz, conn, dofs, ndof, field=None, elem_scale=None):
    b = np.empty(ndof)
    f = None if field is None else np.ascontiguousarray(field, dtype=np.float64)
    s = None if elem_scale is None else np.ascontiguousarray(elem_scale, dtype=np.float64)
    assert lib().or_assemble_rhs(order, QUAD_PREC[quad], _p(xyz), conn.shape[0], _p(conn), _p(dofs), _p(f),
                                 _p(s), ndof, _p(b)) == 0
    return b


def apply_dirichlet(rowptr, colind, mask, values, b=None):
    m = np.ascontiguousarray(mask, dtype=np.uint8)
    lib().or_apply_dirichlet(rowptr.shape[0] - 1, _p(rowptr), _p(colind), _p(m), _p(values), _p(b))


def spmv(rowptr, colind, values, x):
    y = np.empty(rowptr.shape[0] - 1)
    lib().or_spmv(rowptr.shape[0] - 1, _p(rowptr), _p(colind), _p(values), _p(np.ascontiguousarray(x)), _p(y))
    return y


def cg(rowptr, colind, values, b, rtol=1e-10, maxit=10000, precond=1, x0=None):
    x = np.zeros_like(b) if x0 is None else x0.copy()
    it = ctypes.c_int()
    rr = ctypes.c_double()
    rc = lib().or_cg(rowptr.shape[0] - 1, _p(rowptr), _p(colind), _p(values), _p(b), _p(x), rtol, maxit, precond,
                     ctypes.byref(it), ctypes.byref(rr))
    return x, it.value, rr.value, rc


def adjoint_grad(order, quad, xyz, conn, dofs, u, lam):
    g = np.empty(conn.shape[0])
    assert lib().or_adjoint_grad(order, QUAD_PREC[quad], _p(xyz), conn.shape[0], _p(conn), _p(dofs),
                                 _p(np.ascontiguousarray(u)), _p(np.ascontiguousarray(lam)), _p(g)) == 0
    return g


def full_operator(op, order, quad, xyz, conn, coeff=None, c=1.0, edge_rule="lex"):
    """Everything the reference builds for one bilinear form: dofs, pattern, values."""
    n_nodes = xyz.shape[0]
    ee = None
    ndof = n_nodes
    if order == 2:
        en, ee = edges(n_nodes, conn, edge_rule)
        ndof = n_nodes + en.shape[0]
    dofs = elem_dofs(order, n_nodes, conn, ee)
    rp, ci = pattern(order, ndof, dofs)
    vals = assemble(op, order, quad, xyz, conn, dofs, rp, ci, coeff, c)
    return dofs, rp, ci, vals


# ----------------------------------------------------------------------------
# Boundary-face Lagrange operator (opLA3dA) and the saddle system
# ----------------------------------------------------------------------------

def tri_rule(quad: int):
    Y = np.empty((6, 2))
    W = np.empty(6)
    n = lib().or_tri_rule(FACE_QUAD_PREC[quad], _p(Y), _p(W))
    return Y[:n].copy(), W[:n].copy()


TEST_BASIS = {0: 1, 1: 3, 2: 6}  # test functions per boundary triangle (fePr2d<0/1/2>)
TRI_EDGES = np.array([[0, 1], [1, 2], [2, 0]])  # face-local edges of the P2 test basis


def face_matrix(order, quad, xyz, nodes4, lf, test_order=1):
    nb = 4 if order == 1 else 10
    nt = TEST_BASIS[test_order]
    mat = np.empty(nt * nb)
    nodes4 = np.ascontiguousarray(nodes4, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    assert lib().or_face_matrix(order, test_order, FACE_QUAD_PREC[quad], _p(xyz), _p(nodes4), lf, _p(mat)) == 0
    return mat.reshape(nt, nb)  # [test basis a, field basis i]


def boundary_faces(conn, tris=None):
    """(element, local face) of every face with one incident tet, in element then
    local-face order (the loop order of the reference's builder over grid3d and
    localMatrixLA3d::matrix); with `tris` (k x 3 node ids), only the faces that
    are among them (the boundary triangles whose geoIds the test field keeps)."""
    conn = np.asarray(conn)
    tri = conn[:, FACE_PTS].reshape(-1, 3)
    key = np.sort(tri, axis=1)
    order = np.lexsort((key[:, 2], key[:, 1], key[:, 0]))
    ks = key[order]
    head = np.ones(len(ks), dtype=bool)
    head[1:] = np.any(ks[1:] != ks[:-1], axis=1)
    run = np.cumsum(head) - 1
    counts = np.bincount(run) if len(run) else np.zeros(0, dtype=np.int64)
    if counts.max(initial=0) > 2:
        raise ValueError("a face is shared by more than two tets")
    cnt = np.empty(len(ks), dtype=np.int64)
    cnt[order] = counts[run]
    idx = np.nonzero(cnt == 1)[0]
    if tris is not None:
        want = {tuple(t) for t in np.sort(np.asarray(tris), axis=1).tolist()}
        idx = np.array([i for i in idx if tuple(key[i].tolist()) in want], dtype=np.int64)
    return (idx // 4).astype(np.int32), (idx % 4).astype(np.int32)


def lagrange(order, quad, xyz, conn, dofs, ndof, tris=None, faces=None, test_order=1, edge_rule="lex"):
    """B of opLA3dA with P1 (test_order 1), P0 (0) or P2 (2) multipliers on the
    boundary triangles.

    P1 multipliers: the nodes of the selected boundary faces, numbered by
    ascending node id (meshDoctor2d.hpp:339-500 compacts the boundary grid's
    nodes in that order; dofMapStatic2d.hpp:1166-1380 numbers the active
    vertices in that order).  P0 multipliers: one per selected face, numbered in
    the boundary grid's element order -- the order of `tris` when given (the
    Gmsh triangles' order, whose ids the boundary elements keep,
    meshInit3d.hpp:400-430), else the face order.  P2 multipliers: the P1 ones,
    then one per edge of the selected faces in the boundary grid's edge order
    (connect2d.hpp:336-451, kept by dofMapStatic2d.hpp:1166-1380): under
    pMapItem ("lex") (min node, max node) order; under pMapItemShare on one rank
    ("first") the order of first appearance over every boundary triangle, in the
    grid's element order (the faces' own, element then local face) and local
    edges (1,2), (2,3), (3,1) of the triangle's nodes, stored as connect3d.hpp
    stores the face (faceToPoint order, connect3dTest2.log).  Rows = multipliers, columns =
    field dofs; every face contributes its full local block, zeros included
    (traitsMatrixBuilder.hpp:363-441 inserts the whole block), summed in
    element, local-face, test-basis, field-basis order.  `faces` = (face_elem,
    face_local) from boundary_faces, to skip that search.  Returns (lam_item,
    rowptr, colind, values, face_elem, face_local), lam_item = the node (P1) or
    the face index (P0) of each multiplier."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    nb = dofs.shape[1]
    fe, fl = boundary_faces(conn, tris) if faces is None else faces
    nf = fe.shape[0]
    nt = TEST_BASIS[test_order]
    mats = np.empty((nf, nt, nb))
    if nf:
        assert lib().or_face_matrices(order, test_order, FACE_QUAD_PREC[quad], _p(xyz), nf, _p(conn), _p(fe),
                                      _p(fl), _p(mats)) == 0
    fnodes = conn[fe[:, None], FACE_PTS[fl]] if nf else np.zeros((0, 3), np.int32)
    if test_order in (1, 2):
        lam_node = np.unique(fnodes).astype(np.int32)
        lam_of = np.full(xyz.shape[0], -1, dtype=np.int64)
        lam_of[lam_node] = np.arange(lam_node.shape[0])
        face_rows = lam_of[fnodes]
        if test_order == 2:
            ends = np.sort(fnodes[:, TRI_EDGES], axis=2).astype(np.int64)  # nf x 3 x 2
            ekey = ends[:, :, 0] * xyz.shape[0] + ends[:, :, 1]
            uedge = np.unique(ekey)
            if edge_rule == "first":  # first appearance over every boundary triangle
                ae, al = boundary_faces(conn)
                an = conn[ae[:, None], FACE_PTS[al]]
                aends = np.sort(an[:, TRI_EDGES], axis=2).astype(np.int64)
                akey = (aends[:, :, 0] * xyz.shape[0] + aends[:, :, 1]).reshape(-1)
                _, first = np.unique(akey, return_index=True)
                rank_of = dict(zip(akey[np.sort(first)].tolist(), range(len(first))))
                uedge = np.array(sorted(uedge.tolist(), key=lambda k: rank_of[k]), dtype=np.int64)
            pos = {k: i for i, k in enumerate(uedge.tolist())}
            erow = np.array([pos[k] for k in ekey.reshape(-1).tolist()], dtype=np.int64).reshape(ekey.shape)
            face_rows = np.concatenate([face_rows, len(lam_node) + erow], axis=1)
            lam_node = np.concatenate([lam_node, np.full(len(uedge), -1, dtype=np.int32)])
    else:
        if tris is None:
            rank = np.arange(nf)
        else:
            pos = {tuple(t): k for k, t in enumerate(np.sort(np.asarray(tris), axis=1).tolist())}
            rank = np.array([pos[tuple(t)] for t in np.sort(fnodes, axis=1).tolist()], dtype=np.int64)
        lam_node = np.empty(nf, dtype=np.int32)
        lam_node[rank] = np.arange(nf)  # the face carrying each multiplier
        face_rows = rank[:, None]
    rows = np.broadcast_to(face_rows[:, :, None], (nf, nt, nb)).reshape(-1)
    cols = np.broadcast_to(dofs[fe][:, None, :], (nf, nt, nb)).reshape(-1).astype(np.int64)
    key = rows * ndof + cols
    ukey, pos = np.unique(key, return_inverse=True)
    vals = np.zeros(ukey.shape[0])
    np.add.at(vals, pos.reshape(-1), mats.reshape(-1))  # sequential: insertion order
    nl = lam_node.shape[0]
    rowptr = np.zeros(nl + 1, dtype=np.int32)
    np.add.at(rowptr, (ukey // ndof) + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    colind = (ukey % ndof).astype(np.int32)
    return lam_node, rowptr, colind, vals, fe, fl


def mtm(b_rowptr, b_colind, b_vals, ndof):
    """M^T M of a CSR M (here B): the structural product pattern (every pair of
    entries of a row couples, zeros kept, as EpetraExt::MatrixMatrix::Multiply
    builds it for epetraSaddleAssembler::setMTM) with values summed over the rows
    in ascending order.  Returns (rowptr, colind, values) over ndof rows."""
    nl = b_rowptr.shape[0] - 1
    I, J, V = [], [], []
    for l in range(nl):
        c = b_colind[b_rowptr[l]:b_rowptr[l + 1]].astype(np.int64)
        v = b_vals[b_rowptr[l]:b_rowptr[l + 1]]
        I.append(np.repeat(c, len(c)))
        J.append(np.tile(c, len(c)))
        V.append(np.outer(v, v).reshape(-1))
    if not I:
        return np.zeros(ndof + 1, np.int32), np.zeros(0, np.int32), np.zeros(0)
    I, J, V = np.concatenate(I), np.concatenate(J), np.concatenate(V)
    key = I * ndof + J
    ukey, pos = np.unique(key, return_inverse=True)
    vals = np.zeros(len(ukey))
    np.add.at(vals, pos.reshape(-1), V)  # sequential: ascending multiplier row
    rowptr = np.zeros(ndof + 1, dtype=np.int64)
    np.add.at(rowptr, ukey // ndof + 1, 1)
    return np.cumsum(rowptr).astype(np.int32), (ukey % ndof).astype(np.int32), vals


def mmt(b_rowptr, b_colind, b_vals, ndof):
    """M M^T of a CSR M (here B, n_multipliers rows): the structural product
    pattern (every pair of entries of a column couples, zeros kept; setMMT) with
    values summed over the columns in ascending order."""
    nl = b_rowptr.shape[0] - 1
    brow = np.repeat(np.arange(nl), np.diff(b_rowptr))
    order = np.lexsort((brow, b_colind))  # entries by column, then row
    t_ptr = np.concatenate([[0], np.cumsum(np.bincount(b_colind, minlength=ndof))])
    I, J, V = [], [], []
    for c in range(ndof):
        ks = order[t_ptr[c]:t_ptr[c + 1]]
        if len(ks) == 0:
            continue
        r = brow[ks].astype(np.int64)
        v = b_vals[ks]
        I.append(np.repeat(r, len(r)))
        J.append(np.tile(r, len(r)))
        V.append(np.outer(v, v).reshape(-1))
    if not I:
        return np.zeros(nl + 1, np.int32), np.zeros(0, np.int32), np.zeros(0)
    I, J, V = np.concatenate(I), np.concatenate(J), np.concatenate(V)
    key = I * max(nl, 1) + J
    ukey, pos = np.unique(key, return_inverse=True)
    vals = np.zeros(len(ukey))
    np.add.at(vals, pos.reshape(-1), V)  # sequential: ascending column
    rowptr = np.zeros(nl + 1, dtype=np.int64)
    np.add.at(rowptr, ukey // max(nl, 1) + 1, 1)
    return np.cumsum(rowptr).astype(np.int32), (ukey % max(nl, 1)).astype(np.int32), vals


def saddle(k_rowptr, k_colind, k_vals, b_rowptr, b_colind, b_vals, ndof, lam_diag=False, eye_field=0.0,
           eye_lam=0.0, with_mtm=False, mtm_scale=0.0, with_mmt=False, mmt_scale=0.0):
    """[K + eye_field I + mtm_scale B^T B, B^T; B, eye_lam I + mmt_scale B B^T]
    over (ndof + n_multipliers) rows, the layout of
    epetraSaddleAssembler::setDiagMatrix(K, field block) plus setSymmMatrix(B,
    multiplier block, field block), setMTM(B, field block, scale), setMMT(B,
    multiplier block, scale) and setEye on the blocks
    (epetraSaddleAssembler.cpp).  The field rows hold the union of K's and
    (with_mtm) B^T B's columns; the multiplier rows B's columns, then the union
    of the diagonal (lam_diag) and (with_mmt) B B^T's columns.  Returns
    (rowptr, colind, values)."""
    nl = b_rowptr.shape[0] - 1
    brow = np.repeat(np.arange(nl), np.diff(b_rowptr))
    order = np.lexsort((brow, b_colind))  # B^T rows: by field column, then multiplier
    t_cnt = np.bincount(b_colind, minlength=ndof)
    t_ptr = np.concatenate([[0], np.cumsum(t_cnt)])
    t_col = ndof + brow[order]
    t_val = b_vals[order]
    if with_mtm:
        m_rp, m_ci, m_v = mtm(b_rowptr, b_colind, b_vals, ndof)
    rows_c, rows_v = [], []
    for r in range(ndof):
        k0, k1 = k_rowptr[r], k_rowptr[r + 1]
        acc = {int(c): float(v) for c, v in zip(k_colind[k0:k1], k_vals[k0:k1])}
        if with_mtm:
            for c, v in zip(m_ci[m_rp[r]:m_rp[r + 1]], m_v[m_rp[r]:m_rp[r + 1]]):
                acc[int(c)] = acc.get(int(c), 0.0) + mtm_scale * v
        if r in acc:
            acc[r] += eye_field
        cols = sorted(acc)
        rows_c.append(np.concatenate([np.array(cols, dtype=np.int64), t_col[t_ptr[r]:t_ptr[r + 1]]]))
        rows_v.append(np.concatenate([np.array([acc[c] for c in cols]), t_val[t_ptr[r]:t_ptr[r + 1]]]))
    if with_mmt:
        p_rp, p_ci, p_v = mmt(b_rowptr, b_colind, b_vals, ndof)
    for l in range(nl):
        c = b_colind[b_rowptr[l]:b_rowptr[l + 1]].astype(np.int64)
        v = np.asarray(b_vals[b_rowptr[l]:b_rowptr[l + 1]], dtype=np.float64)
        acc = {}
        if lam_diag:
            acc[l] = eye_lam
        if with_mmt:
            for cc, vv in zip(p_ci[p_rp[l]:p_rp[l + 1]], p_v[p_rp[l]:p_rp[l + 1]]):
                acc[int(cc)] = acc.get(int(cc), 0.0) + mmt_scale * vv
        lc = sorted(acc)
        rows_c.append(np.concatenate([c, ndof + np.array(lc, dtype=np.int64)]))
        rows_v.append(np.concatenate([v, np.array([acc[x] for x in lc], dtype=np.float64)]))
    lens = [len(c) for c in rows_c]
    rowptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    colind = np.concatenate(rows_c).astype(np.int32) if rows_c else np.zeros(0, np.int32)
    values = np.concatenate(rows_v).astype(np.float64) if rows_v else np.zeros(0)
    return rowptr, colind, values


def csr_matvec(rowptr, colind, values, x):
    """y = A x for a CSR matrix of any shape (plain sums in row order)."""
    rows = np.repeat(np.arange(rowptr.shape[0] - 1), np.diff(rowptr))
    return np.bincount(rows, weights=values * np.asarray(x)[colind], minlength=rowptr.shape[0] - 1)
