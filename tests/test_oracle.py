"""CPU checks of the oracle itself: quadrature exactness, basis, analytic element
matrices, and the golden data parsed from the reference's own tests."""
import json
import math
import os

import numpy as np
import pytest

import oracle as orc
from morganapublic_gb300 import meshgen

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def monomial_integral(a, b, c):
    """int over the reference tet of x^a y^b z^c = a! b! c! / (a+b+c+3)!"""
    return math.factorial(a) * math.factorial(b) * math.factorial(c) / math.factorial(a + b + c + 3)


@pytest.mark.parametrize("quad,degree,tol", [(1, 1, 1e-15), (4, 2, 1e-15), (15, 5, 1e-15), (64, 7, 2e-10)])
def test_quadrature_exactness(quad, degree, tol):
    Y, W = orc.quad_rule(quad)
    assert abs(W.sum() - 1.0 / 6.0) < tol
    for a in range(degree + 1):
        for b in range(degree + 1 - a):
            for c in range(degree + 1 - a - b):
                q = np.sum(W * Y[:, 0] ** a * Y[:, 1] ** b * Y[:, 2] ** c)
                assert abs(q - monomial_integral(a, b, c)) < tol, (a, b, c)


def test_basis_partition_and_nodes():
    import ctypes
    L = orc.lib()
    # P2 reference nodes (fePr3d.hpp getRefNode order)
    ref = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [.5, 0, 0], [.5, .5, 0], [0, .5, 0],
                    [0, 0, .5], [.5, 0, .5], [0, .5, .5]], dtype=np.float64)
    for order, nb in ((1, 4), (2, 10)):
        for k in range(nb):
            v = np.empty(nb)
            L.or_basis_eval(order, ref[k].ctypes.data, v.ctypes.data)
            e = np.zeros(nb)
            e[k] = 1.0
            assert np.allclose(v, e, atol=1e-15)
        y = np.array([0.1, 0.2, 0.3])
        v = np.empty(nb)
        gx, gy, gz = np.empty(nb), np.empty(nb), np.empty(nb)
        L.or_basis_eval(order, y.ctypes.data, v.ctypes.data)
        L.or_basis_grad(order, y.ctypes.data, gx.ctypes.data, gy.ctypes.data, gz.ctypes.data)
        assert abs(v.sum() - 1) < 1e-15
        assert abs(gx.sum()) < 1e-14 and abs(gy.sum()) < 1e-14 and abs(gz.sum()) < 1e-14
    del ctypes


def test_reference_tet_p1_matrices():
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    nodes = np.arange(4, dtype=np.int32)
    K = orc.local_matrix("stiff_kappa", 1, 4, xyz, nodes, kappa=1.0)
    Kex = np.array([[3, -1, -1, -1], [-1, 1, 0, 0], [-1, 0, 1, 0], [-1, 0, 0, 1]]) / 6.0
    assert np.allclose(K, Kex, atol=1e-15)
    M = orc.local_matrix("mass", 1, 4, xyz, nodes)
    assert np.allclose(M, (np.ones((4, 4)) + np.eye(4)) / 120.0, atol=1e-16)
    K12 = orc.local_matrix("stiff_kappa", 1, 4, xyz, nodes, kappa=12.0)
    assert np.allclose(K12, 12 * Kex, atol=1e-14)
    F = orc.local_matrix("stiff_const", 1, 4, xyz, nodes, c=2.5)
    assert np.allclose(F, 2.5 * Kex, atol=1e-15)


def test_p2_element_properties():
    m = meshgen.kuhn_cube(2, jitter=0.2, seed=5)
    for e in range(0, 48, 7):
        nodes = m.conn[e]
        K = orc.local_matrix("stiff_kappa", 2, 15, m.xyz, nodes, kappa=1.7)
        M = orc.local_matrix("mass", 2, 15, m.xyz, nodes)
        vol = orc.lib().or_element_det(m.xyz.ctypes.data, nodes.ctypes.data) / 6.0
        assert np.allclose(K, K.T, atol=1e-13)
        assert np.allclose(K.sum(axis=0), 0.0, atol=1e-12)
        assert abs(M.sum() - vol) < 1e-15
        assert np.all(np.linalg.eigvalsh(M) > 0)


def test_patch_test_linear_field():
    """Interior rows of K annihilate a linear field (patch test)."""
    m = meshgen.kuhn_cube(4, jitter=0.2, seed=3, permute=True)
    dofs, rp, ci, vals = orc.full_operator("stiff_kappa", 1, 4, m.xyz, m.conn, coeff=np.ones(len(m.conn)))
    u = 1.0 + 2.0 * m.xyz[:, 0] - 0.5 * m.xyz[:, 1] + 3.0 * m.xyz[:, 2]
    r = orc.spmv(rp, ci, vals, u)
    assert np.max(np.abs(r[~m.boundary])) < 1e-12
    # row sums are zero for the stiffness and sum(M) is the cube volume
    assert np.max(np.abs(orc.spmv(rp, ci, vals, np.ones(len(u))))) < 1e-12
    _, rp2, ci2, mv = orc.full_operator("mass", 1, 4, m.xyz, m.conn)
    assert abs(mv.sum() - 1.0) < 1e-13
    _, rp3, ci3, mv2 = orc.full_operator("mass", 2, 15, m.xyz, m.conn)
    assert abs(mv2.sum() - 1.0) < 1e-13


def test_golden_mignon_counts():
    """Edge and dof counts of the reference's mignon3dC mesh match its dofMap logs."""
    g = json.load(open(os.path.join(GOLDEN, "mignon3dC.json")))
    counts = json.load(open(os.path.join(GOLDEN, "dofmap_counts.json")))
    xyz = np.array(g["nodes"], dtype=np.float64)
    conn = np.array(g["tets_1based"], dtype=np.int32) - 1
    assert conn.shape == (8, 4)
    rc, mn, bad = orc.check_jacobian(xyz, conn)
    assert rc == 0 and mn > 0
    for rule in ("lex", "first"):
        en, ee = orc.edges(len(xyz), conn, rule)
        assert len(xyz) == counts["P1"]
        assert len(xyz) + len(en) == counts["P2"] == counts["P2_b"]
        assert len(conn) == counts["P0"]


def test_golden_local_edge_enumeration():
    """connect3dTest2.log: one tet (local nodes 1..4) enumerates its edges in lid
    order (1,2),(2,3),(3,1),(1,4),(2,4),(3,4) -- the first-appearance rule."""
    g = json.load(open(os.path.join(GOLDEN, "connect3d_edges.json")))
    xyz = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0.5, 0.5, 1]], dtype=np.float64)
    conn = np.array([[0, 1, 2, 3]], dtype=np.int32)
    en, ee = orc.edges(4, conn, "first")
    assert ee[0].tolist() == [l - 1 for l in g["lids"]]
    assert (en + 1).tolist() == g["edge_nodes_local_1based"]


def test_edge_rules_on_cube():
    m = meshgen.kuhn_cube(3, permute=True, seed=11)
    en_lex, ee_lex = orc.edges(len(m.xyz), m.conn, "lex")
    en_fa, ee_fa = orc.edges(len(m.xyz), m.conn, "first")
    # same edge set, lex numbering sorted by (min, max)
    key = np.sort(en_lex, axis=1)
    order = np.lexsort((key[:, 1], key[:, 0]))
    assert np.array_equal(order, np.arange(len(key)))
    # first-appearance: the edges of element 0 are 0..5 in local order
    assert ee_fa[0].tolist() == [0, 1, 2, 3, 4, 5]
    assert set(map(tuple, np.sort(en_fa, axis=1))) == set(map(tuple, key))
    # nE for a Kuhn cube: 3 n (n+1)^2 axis + 3 n^2 (n+1) face + n^3 body diagonals
    n = 3
    assert len(en_lex) == 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3


def test_cg_oracle_converges():
    m = meshgen.kuhn_cube(5, jitter=0.2, seed=2)
    kappa = meshgen.lognormal(len(m.conn), 1.0, 7)
    dofs, rp, ci, K = orc.full_operator("stiff_kappa", 1, 4, m.xyz, m.conn, coeff=kappa)
    b = orc.assemble_rhs(1, 4, m.xyz, m.conn, dofs, len(m.xyz))
    orc.apply_dirichlet(rp, ci, m.boundary, K, b)
    x, it, rr, rc = orc.cg(rp, ci, K, b, rtol=1e-12)
    assert rc == 0 and rr <= 1e-12
    r = b - orc.spmv(rp, ci, K, x)
    assert np.linalg.norm(r) <= 1e-11 * np.linalg.norm(b)


# ---------------------------------------------------------------------------
# The oracle against the reference's own code: tests/golden/ref_elements.npz
# holds quadrature cards and element matrices computed by the reference's
# compiled sources (intStaticCards, polyCards via the feStatic iterators,
# geoMapInterface, tensor3d), driven through the opEL3dA/F/G/M integrands and the
# integratorOEL3d_STD loop (oracle/ref, made by tests/golden/make_ref_elements.py).
REF_OPS = ["stiff_kappa", "stiff_const", "mass", "mass_coeff"]
QUAD_OF_PREC = {1: 1, 2: 4, 3: 15, 4: 64}


def _ref_fixture():
    return np.load(os.path.join(GOLDEN, "ref_elements.npz"))


@pytest.mark.parametrize("prec", [1, 2, 3, 4])
def test_quadrature_cards_equal_reference_code(prec):
    d = _ref_fixture()
    Y, W = orc.quad_rule(QUAD_OF_PREC[prec])
    assert np.array_equal(Y, d[f"card{prec}_Y"]) and np.array_equal(W, d[f"card{prec}_W"])


@pytest.mark.parametrize("op", REF_OPS)
@pytest.mark.parametrize("order", [1, 2])
def test_element_matrices_equal_reference_code(op, order):
    """Bit for bit: the oracle restates the reference's arithmetic in the same
    order (built without FP contraction, as the reference code was)."""
    d = _ref_fixture()
    xyz, kappa, c = d["xyz"], d["kappa"], float(d["c"])
    nodes = np.arange(4, dtype=np.int32)
    for prec in (1, 2, 3, 4):
        ref = d[f"m_{op}_{order}_{prec}"]
        for t in range(len(xyz)):
            got = orc.local_matrix(op, order, QUAD_OF_PREC[prec], np.ascontiguousarray(xyz[t]), nodes, kappa[t], c)
            assert np.array_equal(got, ref[t]), (op, order, prec, t, np.max(np.abs(got - ref[t])))
