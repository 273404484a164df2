"""Boundary-face Lagrange operator (opLA3dA) and the saddle matrix, CPU side.

The host half of mg_lagrange (boundary faces, multiplier numbering, the
patterns of B and [K B^T; B 0], the gather maps) runs through the C ABI
without a device and is compared with the oracle bit for bit.  The per-face
arithmetic of the kernel (mg_lagrange.cuh) is compiled for the host by
tests/lagrange/face_check.cpp and run through the exported gather maps, which
is the data flow of the two kernels, against the oracle's values.

The reference's own tests for this operator (operatorLA3dTest1.cpp) print
their results and hold no expected values, so the oracle is pinned here by
properties: the triangle cards integrate monomials exactly to their degree,
the rows of B sum to the integral of each multiplier's hat function (the field
basis is a partition of unity), and the P1 x P1 block is the face mass matrix
area/12 (1 + delta) under a card exact for degree 2."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import morganapublic_gb300 as mg
import oracle as orc
from helpers import row_scaled_err
from morganapublic_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CARDS = [1, 3, 4, 6]
DEGREE = {1: 1, 3: 2, 4: 3, 6: 4}


@pytest.fixture(scope="module")
def face_lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("face") / "libface_check.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-Wall", "-Werror",
                    "-I" + os.path.join(ROOT, "morganapublic_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "lagrange", "face_check.cpp"), "-o", out], check=True)
    L = ctypes.CDLL(out)
    P = ctypes.c_void_p
    L.face_check_matrices.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_int64, P, P, P, P]
    return L


def _p(a):
    return a.ctypes.data


def kernel_face_matrices(face_lib, order, quad, xyz, conn, fe, fl, test_order=1):
    nb = 4 if order == 1 else 10
    out = np.empty((len(fe), orc.TEST_BASIS[test_order], nb))
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    fe = np.ascontiguousarray(fe, dtype=np.int32)
    fl = np.ascontiguousarray(fl, dtype=np.int32)
    assert face_lib.face_check_matrices(order, test_order, quad, _p(xyz), len(fe), _p(conn), _p(fe), _p(fl),
                                        _p(out)) == 0
    return out


def _mesh(n, order, seed=3):
    m = meshgen.kuhn_cube(n, jitter=0.2, seed=seed, permute=True)
    mesh = mg.Mesh(m.xyz, m.conn, order=order)
    return m, mesh, mg.MatrixBuilder(mesh)


# --------------------------------------------------------------- oracle pins --
@pytest.mark.parametrize("quad", CARDS)
def test_triangle_cards_exact_to_their_degree(quad):
    """int over the reference triangle of x^i y^j = i! j! / (i + j + 2)!"""
    from math import factorial
    Y, W = orc.tri_rule(quad)
    assert abs(W.sum() - 0.5) < 1e-15
    for i in range(DEGREE[quad] + 1):
        for j in range(DEGREE[quad] + 1 - i):
            exact = factorial(i) * factorial(j) / factorial(i + j + 2)
            assert abs(np.sum(W * Y[:, 0] ** i * Y[:, 1] ** j) - exact) < 1e-15, (i, j)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("quad", CARDS)
def test_oracle_rows_sum_to_hat_integrals(order, quad):
    m, mesh, b = _mesh(3, order)
    dofs = mesh.elem_dofs()
    lam, rp, ci, v, fe, fl = orc.lagrange(order, quad, m.xyz, m.conn, dofs, b.ndof)
    fn = m.conn[fe[:, None], orc.FACE_PTS[fl]]
    P = m.xyz[fn]
    area = 0.5 * np.linalg.norm(np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), axis=1)
    want = np.zeros(len(lam))
    np.add.at(want, np.searchsorted(lam, fn).reshape(-1), np.repeat(area / 3, 3))
    assert np.abs(np.add.reduceat(v, rp[:-1]) - want).max() < 1e-15
    assert abs(area.sum() - 6.0) < 1e-12  # the unit cube's surface


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("quad", CARDS)
def test_oracle_p0_rows_are_face_areas(order, quad):
    """P0 multipliers: row f of B holds int_f phi_i, which sums to the face area;
    with P1 fields every face vertex gets area / 3 (degree 1, exact for every card)."""
    m, mesh, b = _mesh(3, order)
    dofs = mesh.elem_dofs()
    lam, rp, ci, v, fe, fl = orc.lagrange(order, quad, m.xyz, m.conn, dofs, b.ndof, test_order=0)
    assert np.array_equal(lam, np.arange(len(fe)))  # face order without a triangle list
    fn = m.conn[fe[:, None], orc.FACE_PTS[fl]]
    P = m.xyz[fn]
    area = 0.5 * np.linalg.norm(np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), axis=1)
    assert np.abs(np.add.reduceat(v, rp[:-1]) - area).max() < 1e-15
    if order == 1:
        for f in range(len(fe)):
            row = dict(zip(ci[rp[f]:rp[f + 1]], v[rp[f]:rp[f + 1]]))
            for node in fn[f]:
                assert abs(row[node] - area[f] / 3) < 1e-15


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("quad", [3, 4, 6])
def test_oracle_p2_rows_integrate_the_test_functions(order, quad):
    """P2 multipliers: row a of B sums to int psi_a (the field basis is a partition
    of unity): 0 for every vertex function l (2 l - 1), area / 3 per face for an
    edge function 4 l_p l_q (degree 2: exact for the cards of 3 points and up)."""
    m, mesh, b = _mesh(3, order)
    dofs = mesh.elem_dofs()
    lam, rp, ci, v, fe, fl = orc.lagrange(order, quad, m.xyz, m.conn, dofs, b.ndof, test_order=2)
    nv = int((lam >= 0).sum())
    fn = m.conn[fe[:, None], orc.FACE_PTS[fl]]
    P = m.xyz[fn]
    area = 0.5 * np.linalg.norm(np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), axis=1)
    rows = np.add.reduceat(v, rp[:-1])
    assert np.abs(rows[:nv]).max() < 1e-15
    ends = np.sort(fn[:, orc.TRI_EDGES], axis=2)
    keys = ends[:, :, 0].astype(np.int64) * len(m.xyz) + ends[:, :, 1]
    want = np.zeros(len(lam) - nv)
    np.add.at(want, np.searchsorted(np.unique(keys), keys).reshape(-1), np.repeat(area / 3, 3))
    assert np.abs(rows[nv:] - want).max() < 1e-15


def test_oracle_p1_block_is_the_face_mass_matrix():
    m = meshgen.kuhn_cube(2, jitter=0.25, seed=5, permute=False)
    for e in range(len(m.conn)):
        for lf in range(4):
            mat = orc.face_matrix(1, 3, m.xyz, m.conn[e], lf)
            P = m.xyz[m.conn[e][orc.FACE_PTS[lf]]]
            area = 0.5 * np.linalg.norm(np.cross(P[1] - P[0], P[2] - P[0]))
            want = np.zeros((3, 4))
            for a in range(3):
                for bb in range(3):
                    want[a, orc.FACE_PTS[lf][bb]] = area / 12 * (2 if a == bb else 1)
            assert np.abs(mat - want).max() <= 1e-15 * max(area, 1.0)


# ------------------------------------------------------ kernel arithmetic --
@pytest.mark.parametrize("test_order", [1, 0, 2])
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("quad", CARDS)
def test_kernel_face_math_matches_oracle(face_lib, order, quad, test_order):
    m, mesh, b = _mesh(3, order, seed=7)
    fe, fl = orc.boundary_faces(m.conn)
    ref = np.stack([orc.face_matrix(order, quad, m.xyz, m.conn[e], l, test_order) for e, l in zip(fe, fl)])
    got = kernel_face_matrices(face_lib, order, quad, m.xyz, m.conn, fe, fl, test_order)
    scale = np.abs(ref).max(axis=(1, 2), keepdims=True)
    assert np.max(np.abs(got - ref) / scale) < 1e-14


# --------------------------------------------------------- host ABI (no GPU) --
def _tris_on_plane(m, axis, value):
    fe, fl = orc.boundary_faces(m.conn)
    fn = m.conn[fe[:, None], orc.FACE_PTS[fl]]
    on = np.all(np.abs(m.xyz[fn][:, :, axis] - value) < 1e-12, axis=1)
    return fn[on][:, ::-1].copy()  # any vertex order


@pytest.mark.parametrize("products", ["", "mtm", "mmt", "mtm+mmt"])
@pytest.mark.parametrize("test_order", [1, 0, 2])
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("select", [None, "x0", "x0z1"])
@pytest.mark.parametrize("lam_diag", [False, True])
def test_patterns_match_oracle(order, select, lam_diag, test_order, products):
    mtm, mmt = "mtm" in products, "mmt" in products
    m, mesh, b = _mesh(4 if order == 1 else 3, order, seed=11)
    tris = None
    if select == "x0":
        tris = _tris_on_plane(m, 0, 0.0)
    elif select == "x0z1":  # in an order unrelated to the faces': P0 multipliers follow it
        tris = np.concatenate([_tris_on_plane(m, 2, 1.0), _tris_on_plane(m, 0, 0.0)])
        tris = tris[np.random.default_rng(3).permutation(len(tris))]
    lg = mg.LagrangeBuilder(b, tris=tris, lam_diag=lam_diag, test_order=test_order, mtm=mtm, mmt=mmt)
    lam, fe, fl = lg.multipliers()
    (brp, bci), (srp, sci) = lg.pattern()
    dofs = mesh.elem_dofs()
    olam, obrp, obci, obv, ofe, ofl = orc.lagrange(order, 1, m.xyz, m.conn, dofs, b.ndof, tris=tris,
                                                   test_order=test_order)
    if mtm:
        mrp, mci, _ = orc.mtm(obrp, obci, obv, b.ndof)
        assert lg.nnz_mtm == len(mci)
    if mmt:
        prp, pci, _ = orc.mmt(obrp, obci, obv, b.ndof)
        assert lg.nnz_mmt == len(pci)
    assert np.array_equal(fe, ofe) and np.array_equal(fl, ofl)
    assert np.array_equal(lam, olam)
    if test_order == 2:  # edge multipliers: the selected faces' edges in (min, max) order
        fn = m.conn[ofe[:, None], orc.FACE_PTS[ofl]]
        ends = np.unique(np.sort(fn[:, orc.TRI_EDGES], axis=2).reshape(-1, 2), axis=0)
        assert np.array_equal(lg.edge_multipliers(), ends)
    assert np.array_equal(brp, obrp) and np.array_equal(bci, obci)
    rp, ci = b.pattern()
    orp, oci, _ = orc.saddle(rp, ci, np.zeros(len(ci)), obrp, obci, obv, b.ndof, lam_diag=lam_diag, with_mtm=mtm,
                             with_mmt=mmt)
    assert np.array_equal(srp, orp) and np.array_equal(sci, oci)
    if select is not None:
        assert lg.n_faces == len(tris)


@pytest.mark.parametrize("products", ["", "mtm", "mmt", "mtm+mmt"])
@pytest.mark.parametrize("test_order", [1, 0, 2])
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("quad", [1, 6])
def test_kernel_data_flow_matches_oracle(face_lib, order, quad, test_order, products):
    """The two kernels' data flow on the host: face matrices (the kernel's own
    arithmetic), the per-entry gather lists of B, the saddle source map."""
    m, mesh, b = _mesh(4 if order == 1 else 3, order, seed=13)
    mtm, mmt = "mtm" in products, "mmt" in products
    lg = mg.LagrangeBuilder(b, lam_diag=True, test_order=test_order, mtm=mtm, mmt=mmt)
    lam, fe, fl = lg.multipliers()
    (brp, bci), (srp, sci) = lg.pattern()
    bptr, bsrc, ssrc = lg.export_maps()
    fm = kernel_face_matrices(face_lib, order, quad, m.xyz, m.conn, fe, fl, test_order).reshape(-1)
    bv = np.array([np.sum(fm[bsrc[bptr[k]:bptr[k + 1]]]) for k in range(lg.nnz_b)])
    dofs = mesh.elem_dofs()
    _, orp, oci, ov, _, _ = orc.lagrange(order, quad, m.xyz, m.conn, dofs, b.ndof, test_order=test_order)
    assert row_scaled_err(orp, ov, bv) <= 1e-13
    # every face-matrix entry is used exactly once
    assert np.array_equal(np.sort(bsrc), np.arange(len(fe) * orc.TEST_BASIS[test_order] * mesh.nb))
    # saddle values through the source map
    rp, ci = b.pattern()
    kv = np.random.default_rng(1).uniform(-1, 1, len(ci))
    # k_saddle_fill
    bidx = np.clip(-(ssrc.astype(np.int64) + 1), 0, lg.nnz_b - 1)
    sv = np.where(ssrc >= 0, kv[np.maximum(ssrc, 0)], bv[bidx])
    sv[ssrc == np.iinfo(np.int32).min] = -0.25         # eye_lam
    sv[ssrc == np.iinfo(np.int32).min + 1] = 0.0        # B^T B entries outside K
    # k_saddle_eye at each field row's diagonal entry
    nd = b.ndof
    for r in range(nd):
        hit = np.nonzero(sci[srp[r]:srp[r + 1]] == r)[0]
        if len(hit):
            sv[srp[r] + hit[0]] += 0.5
    # k_saddle_products, B^T B then B B^T
    for which, on, scale in (("mtm", mtm, 2.0), ("mmt", mmt, -1.5)):
        if not on:
            continue
        pp, pairs, slot = lg.export_products(which)
        for mm in range(len(slot)):
            pr = pairs[pp[mm]:pp[mm + 1]]
            sv[slot[mm]] += scale * np.sum(bv[pr[:, 0]] * bv[pr[:, 1]])
        assert len(np.unique(slot)) == len(slot)  # one saddle entry per product entry
    orp_s, oci_s, osv = orc.saddle(rp, ci, kv, brp, bci, bv, nd, lam_diag=True, eye_field=0.5, eye_lam=-0.25,
                                   with_mtm=mtm, mtm_scale=2.0, with_mmt=mmt, mmt_scale=-1.5)
    assert np.array_equal(srp, orp_s) and np.array_equal(sci, oci_s)
    assert row_scaled_err(orp_s, osv, sv) <= 1e-14

def test_selected_triangles_errors():
    m, mesh, b = _mesh(3, 1)
    good = _tris_on_plane(m, 0, 0.0)
    interior = np.array([m.conn[0][[0, 1, 2]]])  # a face of some tet; pick one that is interior
    fe, fl = orc.boundary_faces(m.conn)
    bset = {tuple(sorted(t)) for t in m.conn[fe[:, None], orc.FACE_PTS[fl]].tolist()}
    for e in range(len(m.conn)):
        for lf in range(4):
            t = m.conn[e][orc.FACE_PTS[lf]]
            if tuple(sorted(t.tolist())) not in bset:
                interior = t[None, :]
                break
        else:
            continue
        break
    with pytest.raises(mg.MorganaError) as e:
        mg.LagrangeBuilder(b, tris=np.concatenate([good, interior]))
    assert e.value.status == mg.MG_ERR_BAD_MESH
    with pytest.raises(mg.MorganaError) as e:
        mg.LagrangeBuilder(b, tris=np.concatenate([good, good[:1]]))
    assert e.value.status == mg.MG_ERR_INVALID_ARG
    bad = good.copy()
    bad[0, 0] = len(m.xyz)
    with pytest.raises(mg.MorganaError) as e:
        mg.LagrangeBuilder(b, tris=bad)
    assert e.value.status == mg.MG_ERR_INVALID_ARG
    empty = mg.LagrangeBuilder(b, tris=np.zeros((0, 3), dtype=np.int32))
    assert empty.n_faces == 0 and empty.n_multipliers == 0 and empty.nnz_b == 0
    rp, ci = b.pattern()
    assert empty.nnz_saddle == len(ci)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("select", [None, "x0z1"])
def test_p2_multipliers_on_first_numbered_meshes(face_lib, order, select):
    """Under the FIRST rule the edge multipliers follow first appearance over the
    whole boundary grid, also when only some triangles carry multipliers."""
    m = meshgen.kuhn_cube(3, jitter=0.2, seed=17, permute=True)
    mesh = mg.Mesh(m.xyz, m.conn, order=order, edge_rule="first")
    b = mg.MatrixBuilder(mesh)
    tris = None
    if select:
        tris = np.concatenate([_tris_on_plane(m, 2, 1.0), _tris_on_plane(m, 0, 0.0)])
    lg = mg.LagrangeBuilder(b, tris=tris, test_order=2)
    dofs = mesh.elem_dofs()
    lam, rp, ci, v, fe, fl = orc.lagrange(order, 6, m.xyz, m.conn, dofs, b.ndof, tris=tris, test_order=2,
                                          edge_rule="first")
    lex = orc.lagrange(order, 6, m.xyz, m.conn, dofs, b.ndof, tris=tris, test_order=2)
    assert not np.array_equal(ci, lex[2]) or not np.array_equal(rp, lex[1])  # the rule changes the numbering
    (brp, bci), _ = lg.pattern()
    assert np.array_equal(lg.multipliers()[0], lam) and np.array_equal(brp, rp) and np.array_equal(bci, ci)
    # the edge table in multiplier order: first appearance over every boundary face
    ae, al = orc.boundary_faces(m.conn)
    an = m.conn[ae[:, None], orc.FACE_PTS[al]]
    seen, order_all = set(), []
    for t in an.tolist():
        for j in range(3):
            k = tuple(sorted((t[j], t[(j + 1) % 3])))
            if k not in seen:
                seen.add(k)
                order_all.append(k)
    fn = m.conn[fe[:, None], orc.FACE_PTS[fl]]
    mine = {tuple(sorted((t[j], t[(j + 1) % 3]))) for t in fn.tolist() for j in range(3)}
    assert [tuple(e) for e in lg.edge_multipliers().tolist()] == [k for k in order_all if k in mine]
    bptr, bsrc, _ = lg.export_maps()
    fm = kernel_face_matrices(face_lib, order, 6, m.xyz, m.conn, fe, fl, 2).reshape(-1)
    bv = np.array([np.sum(fm[bsrc[bptr[k]:bptr[k + 1]]]) for k in range(lg.nnz_b)])
    assert row_scaled_err(rp, v, bv) <= 1e-13


def test_face_in_three_tets_is_rejected():
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, -1], [0.1, 0.1, 2.0]], dtype=np.float64)
    conn = np.array([[0, 1, 2, 3], [0, 2, 1, 4], [0, 1, 2, 5]], dtype=np.int32)
    b = mg.MatrixBuilder(mg.Mesh(xyz, conn, order=1))
    with pytest.raises(mg.MorganaError) as e:
        mg.LagrangeBuilder(b)
    assert e.value.status == mg.MG_ERR_BAD_MESH


def test_single_tet_all_faces_boundary():
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    conn = np.array([[0, 1, 2, 3]], dtype=np.int32)
    for order in (1, 2):
        mesh = mg.Mesh(xyz, conn, order=order)
        b = mg.MatrixBuilder(mesh)
        lg = mg.LagrangeBuilder(b)
        lam, fe, fl = lg.multipliers()
        assert np.array_equal(lam, [0, 1, 2, 3]) and np.array_equal(fe, [0] * 4) and np.array_equal(fl, range(4))
        assert lg.nnz_b == 4 * mesh.nb  # every multiplier couples to every dof of the tet


def _write_gmsh(path, g):
    """The fixture in the Gmsh 2 layout it was read from (3 tags: physical, geoId, partition)."""
    nodes, tets, tris = g["nodes"], g["tets_1based"], g["triangles_1based"]
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.1 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(nodes))
        for k, x in enumerate(nodes):
            f.write("%d %r %r %r\n" % (k + 1, *x))
        f.write("$EndNodes\n$Elements\n%d\n" % (len(tets) + len(tris)))
        k = 1
        for t, gid in zip(tris, g["triangle_geo_ids"]):
            f.write("%d 2 3 0 %d 0 %d %d %d\n" % (k, gid, *t))
            k += 1
        for t, gid in zip(tets, g["geo_ids"]):
            f.write("%d 4 3 0 %d 0 %d %d %d %d\n" % (k, gid, *t))
            k += 1
        f.write("$EndElements\n")


@pytest.mark.parametrize("test_order", [0, 1, 2])
def test_reference_mesh_mignon3dB_multipliers_on_geo_id_2(face_lib, tmp_path, test_order):
    """The configuration of the reference's localMatrixLA3dTest1: mignon3dB.msh,
    P1 field, multipliers on the triangles of geoId 2 (fePr2d<0> there),
    triangle card of precision 2; here also P1 / P2 multipliers."""
    import json
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "mignon3dB.json")))
    p = str(tmp_path / "mignon3dB.msh")
    _write_gmsh(p, g)
    mesh = mg.Mesh.load_gmsh(p, order=1)
    tris, geo = mesh.triangles()
    assert np.array_equal(tris, np.array(g["triangles_1based"]) - 1)
    assert np.array_equal(geo, g["triangle_geo_ids"])
    sel, _ = mesh.triangles(geo_ids=[2])
    assert len(sel) == 4
    b = mg.MatrixBuilder(mesh)
    lg = mg.LagrangeBuilder(b, tris=sel, test_order=test_order)
    xyz, conn = mesh.geometry()
    dofs = mesh.elem_dofs()
    lam, rp, ci, ref, fe, fl = orc.lagrange(1, 3, xyz, conn, dofs, b.ndof, tris=sel, test_order=test_order)
    glam, gfe, gfl = lg.multipliers()
    (brp, bci), _ = lg.pattern()
    assert np.array_equal(glam, lam) and np.array_equal(gfe, fe) and np.array_equal(brp, rp)
    assert np.array_equal(bci, ci)
    if test_order == 0:  # one multiplier per triangle, in file order
        fn = np.sort(conn[fe[:, None], orc.FACE_PTS[fl]], axis=1)
        assert np.array_equal(fn[glam], np.sort(sel, axis=1))
    bptr, bsrc, _ = lg.export_maps()
    fm = kernel_face_matrices(face_lib, 1, 3, xyz, conn, gfe, gfl, test_order).reshape(-1)
    bv = np.array([np.sum(fm[bsrc[bptr[k]:bptr[k + 1]]]) for k in range(lg.nnz_b)])
    assert row_scaled_err(rp, ref, bv) <= 1e-13


@pytest.mark.parametrize("test_order", [0, 1, 2])
@pytest.mark.parametrize("order", [1, 2])
def test_edge_meshes_with_every_option(order, test_order):
    """No tets (every row of K empty) and a single tet beside an unreferenced
    node: patterns against the oracle with the diagonal, B^T B and B B^T."""
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [5, 5, 5]], dtype=np.float64)
    for conn in (np.zeros((0, 4), np.int32), np.array([[0, 1, 2, 3]], np.int32)):
        mesh = mg.Mesh(xyz, conn, order=order)
        b = mg.MatrixBuilder(mesh)
        lg = mg.LagrangeBuilder(b, test_order=test_order, lam_diag=True, mtm=True, mmt=True)
        (brp, bci), (srp, sci) = lg.pattern()
        if len(conn) == 0:
            assert lg.n_faces == 0 and lg.n_multipliers == 0 and lg.nnz_b == 0 and lg.nnz_saddle == 0
            continue
        dofs = mesh.elem_dofs()
        lam, rp_o, ci_o, v_o, fe, fl = orc.lagrange(order, 1, xyz, conn, dofs, b.ndof, test_order=test_order)
        assert np.array_equal(lg.multipliers()[0], lam) and 4 not in lam  # the unreferenced node carries none
        assert np.array_equal(brp, rp_o) and np.array_equal(bci, ci_o)
        rp, ci = b.pattern()
        orp, oci, _ = orc.saddle(rp, ci, np.zeros(len(ci)), rp_o, ci_o, v_o, b.ndof, lam_diag=True, with_mtm=True,
                                 with_mmt=True)
        assert np.array_equal(srp, orp) and np.array_equal(sci, oci)


def test_argument_errors_before_any_device_work():
    """Bad options are refused with MG_ERR_INVALID_ARG (or MG_ERR_UNSUPPORTED)
    before anything touches a device."""
    m, mesh, b = _mesh(2, 1)
    L = mg.lib()
    h = ctypes.c_void_p()
    for test_order, flags in ((3, 0), (-1, 0), (1, 8), (1, -1)):
        assert L.mg_lagrange_build(b._h, test_order, 0, None, flags, ctypes.byref(h)) == mg.MG_ERR_INVALID_ARG
    lg = mg.LagrangeBuilder(b)  # no diagonal, no products in the pattern
    assert L.mg_lagrange_assemble(lg._h, 2, None, None) == mg.MG_ERR_INVALID_ARG  # no 2-point card
    for scales in (mg.SaddleScales(0, 1.0, 0, 0), mg.SaddleScales(0, 0, 1.0, 0), mg.SaddleScales(0, 0, 0, 1.0)):
        assert L.mg_saddle_assemble(lg._h, None, None, ctypes.byref(scales), None, None) == mg.MG_ERR_INVALID_ARG
    assert L.mg_lagrange_export_products(lg._h, 1, None, None, None) == mg.MG_ERR_INVALID_ARG
    assert L.mg_lagrange_build(None, 1, 0, None, 0, ctypes.byref(h)) == mg.MG_ERR_INVALID_ARG
    assert L.mg_lagrange_build(b._h, 1, 3, None, 0, ctypes.byref(h)) == mg.MG_ERR_INVALID_ARG  # count without list
