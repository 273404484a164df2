"""Boundary-face Lagrange operator and saddle matrix on the GPU against the oracle.

B = opLA3dA (P1 multipliers on the boundary triangles x the P1/P2 field) from
mg_lagrange_assemble, the saddle values [K + eI, B^T; B, e'I] from
mg_saddle_assemble, and the products mg_saddle_spmv / mg_lagrange_apply,
each against the oracle at FP64 (1e-12 row-scaled for values, 1e-12 relative
for products).  An end-to-end check solves the saddle system of a Poisson
problem (on the host, from the GPU's values) and compares its field with the
symmetric elimination of the same Dirichlet data: for P1 they agree, because
the multiplier rows pin the boundary values exactly.  This file is collected
last so that a -x run has run every other test first if it fails."""
import numpy as np
import pytest

import morganapublic_gb300 as mg
import oracle as orc
from helpers import row_scaled_err
from morganapublic_gb300 import meshgen

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def _setup(n, order, seed, tris_plane=None, lam_diag=False):
    m = meshgen.kuhn_cube(n, jitter=0.2, seed=seed, permute=True)
    mesh = mg.Mesh(m.xyz, m.conn, order=order)
    b = mg.MatrixBuilder(mesh)
    tris = None
    if tris_plane is not None:
        fe, fl = orc.boundary_faces(m.conn)
        fn = m.conn[fe[:, None], orc.FACE_PTS[fl]]
        axis, value = tris_plane
        tris = fn[np.all(np.abs(m.xyz[fn][:, :, axis] - value) < 1e-12, axis=1)]
    lg = mg.LagrangeBuilder(b, tris=tris, lam_diag=lam_diag)
    return m, mesh, b, lg, tris


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("quad", [1, 3, 4, 6])
def test_b_values_match_oracle(order, quad):
    m, mesh, b, lg, _ = _setup(4 if order == 1 else 3, order, 21)
    got = lg.assemble(quad=quad)
    again = lg.assemble(quad=quad)
    torch.cuda.synchronize()
    dofs = mesh.elem_dofs()
    lam, rp, ci, ref, fe, fl = orc.lagrange(order, quad, m.xyz, m.conn, dofs, b.ndof)
    (brp, bci), _ = lg.pattern()
    assert np.array_equal(brp, rp) and np.array_equal(bci, ci)
    assert row_scaled_err(rp, ref, got.cpu().numpy()) <= 1e-12
    assert torch.equal(got, again)  # deterministic: no atomics


@pytest.mark.parametrize("order", [1, 2])
def test_b_on_selected_triangles(order):
    m, mesh, b, lg, tris = _setup(4 if order == 1 else 3, order, 22, tris_plane=(0, 0.0))
    got = lg.assemble(quad=3).cpu().numpy()
    dofs = mesh.elem_dofs()
    lam, rp, ci, ref, fe, fl = orc.lagrange(order, 3, m.xyz, m.conn, dofs, b.ndof, tris=tris)
    assert lg.n_faces == len(tris) and lg.n_multipliers == len(lam)
    assert row_scaled_err(rp, ref, got) <= 1e-12


@pytest.mark.parametrize("order", [1, 2])
def test_saddle_values_and_products(order):
    m, mesh, b, lg, _ = _setup(4 if order == 1 else 3, order, 23, lam_diag=True)
    kappa = meshgen.lognormal(len(m.conn), 1.0, 23)
    K = b.assemble("stiff_kappa", coeff=kappa, quad=4)
    B = lg.assemble(quad=3)
    S = lg.saddle(K, B, eye_field=0.5, eye_lam=-0.25)
    dofs, rp, ci, kref = orc.full_operator("stiff_kappa", order, 4, m.xyz, m.conn, coeff=kappa)
    _, brp, bci, bref, _, _ = orc.lagrange(order, 3, m.xyz, m.conn, dofs, b.ndof)
    srp, sci, sref = orc.saddle(rp, ci, kref, brp, bci, bref, b.ndof, lam_diag=True, eye_field=0.5,
                                eye_lam=-0.25)
    (_, _), (gsrp, gsci) = lg.pattern()
    assert np.array_equal(gsrp, srp) and np.array_equal(gsci, sci)
    assert row_scaled_err(srp, sref, S.cpu().numpy()) <= 1e-12
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, b.ndof + lg.n_multipliers)
    y = lg.saddle_apply(S, torch.from_numpy(x).cuda()).cpu().numpy()
    yref = orc.csr_matvec(srp, sci, sref, x)
    assert np.abs(y - yref).max() <= 1e-12 * np.abs(yref).max()
    u = rng.uniform(-1, 1, b.ndof)
    g = lg.apply(B, torch.from_numpy(u).cuda()).cpu().numpy()
    gref = orc.csr_matvec(brp, bci, bref, u)
    assert np.abs(g - gref).max() <= 1e-12 * np.abs(gref).max()


def test_saddle_solution_equals_elimination():
    scipy_sparse = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    m, mesh, b, lg, _ = _setup(4, 1, 24)
    K = b.assemble("stiff_const", quad=4)
    B = lg.assemble(quad=3)
    S = lg.saddle(K, B)
    nd, nl = b.ndof, lg.n_multipliers
    (_, _), (srp, sci) = lg.pattern()
    A = scipy_sparse.csr_matrix((S.cpu().numpy(), sci, srp), shape=(nd + nl, nd + nl))
    dofs = mesh.elem_dofs()
    f = orc.assemble_rhs(1, 4, m.xyz, m.conn, dofs, nd)
    uD = 1.0 + m.xyz[:, 0] + 2.0 * m.xyz[:, 1] - m.xyz[:, 2]  # boundary data at the nodes
    g = lg.apply(B, torch.from_numpy(uD).cuda()).cpu().numpy()
    sol = spla.spsolve(A.tocsc(), np.concatenate([f, g]))
    u_saddle = sol[:nd]
    # symmetric elimination of the same data (the library's own build addition)
    _, rp, ci, kv = orc.full_operator("stiff_const", 1, 4, m.xyz, m.conn)
    mask = m.boundary.astype(np.uint8)
    kv = kv.copy()
    rhs = f - orc.csr_matvec(rp, ci, kv, np.where(mask == 1, uD, 0.0))
    orc.apply_dirichlet(rp, ci, mask, kv, rhs)
    rhs[mask == 1] = uD[mask == 1]
    Ke = scipy_sparse.csr_matrix((kv, ci, rp), shape=(nd, nd))
    u_elim = spla.spsolve(Ke.tocsc(), rhs)
    assert np.abs(u_saddle - u_elim).max() <= 1e-9 * np.abs(u_elim).max()
    lam_nodes, _, _ = lg.multipliers()
    assert np.abs(u_saddle[lam_nodes] - uD[lam_nodes]).max() <= 1e-9


def test_empty_selection_gives_k():
    m, mesh, b, _, _ = _setup(3, 1, 25)
    lg = mg.LagrangeBuilder(b, tris=np.zeros((0, 3), dtype=np.int32))
    K = b.assemble("mass", quad=4)
    B = lg.assemble(quad=1)
    assert B.numel() == 0
    S = lg.saddle(K, B)
    assert torch.equal(S, K)


@pytest.mark.parametrize("order", [1, 2])
def test_trilinos_adapters_for_multipliers(tmp_path, order):
    """buildEpetraLagrange / buildTpetraLagrange rows (test doubles of the
    Trilinos classes) and GpuSaddleOperator::Apply against the oracle."""
    import os
    import subprocess
    from morganapublic_gb300 import build as mgbuild
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = os.path.join(root, "tests", "adapter", "adapter_check.cpp")
    lib = mgbuild.build()
    exe = str(tmp_path / "adapter_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(root, "include"),
                    "-I" + os.path.join(root, "tests", "adapter", "mock_trilinos"),
                    "-I" + os.path.join(mgbuild.CUDA_HOME, "include"), src, "-o", exe, lib,
                    "-L" + os.path.join(mgbuild.CUDA_HOME, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.dirname(lib),
                    "-Wl,-rpath," + os.path.join(mgbuild.CUDA_HOME, "lib64")], check=True)
    m = meshgen.kuhn_cube(4 if order == 1 else 3, jitter=0.2, seed=41, permute=True)
    kappa = meshgen.lognormal(len(m.conn), 1.0, 41)
    dofs, rp, ci, kref = orc.full_operator("stiff_kappa", order, 4, m.xyz, m.conn, coeff=kappa)
    ndof = len(rp) - 1
    lam, brp, bci, bref, _, _ = orc.lagrange(order, 1, m.xyz, m.conn, dofs, ndof)
    n = ndof + len(lam)
    x = np.random.default_rng(4).uniform(-1, 1, n)
    with open(tmp_path / "in.bin", "wb") as f:
        np.array([len(m.xyz), len(m.conn), order], dtype=np.int64).tofile(f)
        m.xyz.astype(np.float64).tofile(f)
        m.conn.astype(np.int32).tofile(f)
        kappa.astype(np.float64).tofile(f)
        x.tofile(f)
    subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), "lagrange"], check=True, timeout=300)
    raw = open(tmp_path / "out.bin", "rb").read()
    nl, nz = np.frombuffer(raw[:16], dtype=np.int64)
    off = 16
    rp_g = np.frombuffer(raw[off:off + 4 * (nl + 1)], dtype=np.int32); off += 4 * (nl + 1)
    ci_g = np.frombuffer(raw[off:off + 4 * nz], dtype=np.int32); off += 4 * nz
    va_g = np.frombuffer(raw[off:off + 8 * nz], dtype=np.float64); off += 8 * nz
    y_g = np.frombuffer(raw[off:off + 8 * n], dtype=np.float64)
    assert nl == len(lam) and np.array_equal(rp_g, brp) and np.array_equal(ci_g, bci)
    assert row_scaled_err(brp, bref, va_g) <= 1e-12
    srp, sci, sref = orc.saddle(rp, ci, kref, brp, bci, bref, ndof)
    yref = orc.csr_matvec(srp, sci, sref, x)
    assert np.abs(y_g - yref).max() <= 1e-12 * np.abs(yref).max()


def test_host_buffer_b_equals_device_b():
    m, mesh, b, lg, _ = _setup(3, 2, 26)
    dev = lg.assemble(quad=4).cpu().numpy()
    host = lg.build_crs(quad=4)
    (brp, bci), _ = lg.pattern()
    assert np.array_equal(host.rowptr, brp) and np.array_equal(host.colind, bci)
    assert np.array_equal(host.values, dev)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("quad", [1, 3])
def test_p0_multipliers_match_oracle(order, quad):
    """fePr2d<0> multipliers (one per triangle, numbered in the order of the
    given triangles), as in the reference's localMatrixLA3dTest1."""
    m = meshgen.kuhn_cube(4 if order == 1 else 3, jitter=0.2, seed=27, permute=True)
    mesh = mg.Mesh(m.xyz, m.conn, order=order)
    b = mg.MatrixBuilder(mesh)
    fe, fl = orc.boundary_faces(m.conn)
    fn = m.conn[fe[:, None], orc.FACE_PTS[fl]]
    on = np.all(np.abs(m.xyz[fn][:, :, 0]) < 1e-12, axis=1) | np.all(np.abs(m.xyz[fn][:, :, 2] - 1) < 1e-12,
                                                                     axis=1)
    tris = fn[on][np.random.default_rng(2).permutation(int(on.sum()))]  # x = 0 and z = 1, shuffled
    lg = mg.LagrangeBuilder(b, tris=tris, test_order=0)
    got = lg.assemble(quad=quad)
    again = lg.assemble(quad=quad)
    dofs = mesh.elem_dofs()
    lam, rp, ci, ref, _, _ = orc.lagrange(order, quad, m.xyz, m.conn, dofs, b.ndof, tris=tris, test_order=0)
    (brp, bci), _ = lg.pattern()
    assert lg.n_multipliers == len(tris) and np.array_equal(brp, rp) and np.array_equal(bci, ci)
    assert row_scaled_err(rp, ref, got.cpu().numpy()) <= 1e-12
    assert torch.equal(got, again)


@pytest.mark.parametrize("order", [1, 2])
def test_saddle_with_mtm_matches_oracle(order):
    """setMTM: K + eye_field I + scale B^T B on the field block (structural
    B^T B pattern merged into K's), the multiplier diagonal, and the products."""
    m, mesh, b, _, _ = _setup(4 if order == 1 else 3, order, 28)
    lg = mg.LagrangeBuilder(b, lam_diag=True, mtm=True)
    kappa = meshgen.lognormal(len(m.conn), 1.0, 28)
    K = b.assemble("stiff_kappa", coeff=kappa, quad=4)
    B = lg.assemble(quad=3)
    S = lg.saddle(K, B, eye_field=0.5, eye_lam=-0.25, mtm_scale=3.0)
    S2 = lg.saddle(K, B, eye_field=0.5, eye_lam=-0.25, mtm_scale=3.0)
    dofs, rp, ci, kref = orc.full_operator("stiff_kappa", order, 4, m.xyz, m.conn, coeff=kappa)
    _, brp, bci, bref, _, _ = orc.lagrange(order, 3, m.xyz, m.conn, dofs, b.ndof)
    srp, sci, sref = orc.saddle(rp, ci, kref, brp, bci, bref, b.ndof, lam_diag=True, eye_field=0.5, eye_lam=-0.25,
                                with_mtm=True, mtm_scale=3.0)
    (_, _), (gsrp, gsci) = lg.pattern()
    assert np.array_equal(gsrp, srp) and np.array_equal(gsci, sci)
    assert row_scaled_err(srp, sref, S.cpu().numpy()) <= 1e-12
    assert torch.equal(S, S2)
    x = np.random.default_rng(6).uniform(-1, 1, b.ndof + lg.n_multipliers)
    y = lg.saddle_apply(S, torch.from_numpy(x).cuda()).cpu().numpy()
    yref = orc.csr_matvec(srp, sci, sref, x)
    assert np.abs(y - yref).max() <= 1e-12 * np.abs(yref).max()


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("quad", [3, 6])
def test_p2_multipliers_match_oracle(order, quad):
    """fePr2d<2> multipliers: the boundary nodes, then the boundary edges in
    (min node, max node) order."""
    m, mesh, b, _, _ = _setup(4 if order == 1 else 3, order, 29)
    lg = mg.LagrangeBuilder(b, test_order=2)
    got = lg.assemble(quad=quad)
    again = lg.assemble(quad=quad)
    dofs = mesh.elem_dofs()
    lam, rp, ci, ref, _, _ = orc.lagrange(order, quad, m.xyz, m.conn, dofs, b.ndof, test_order=2)
    (brp, bci), _ = lg.pattern()
    assert lg.n_multipliers == len(lam) and np.array_equal(brp, rp) and np.array_equal(bci, ci)
    assert row_scaled_err(rp, ref, got.cpu().numpy()) <= 1e-12
    assert torch.equal(got, again)


def test_reference_mesh_mignon3dB_geo_id_2(tmp_path):
    """localMatrixLA3dTest1's configuration on the GPU: mignon3dB.msh, P1 field,
    P0 multipliers on the triangles of geoId 2, triangle card of precision 2."""
    import json
    import os
    from test_lagrange_host import _write_gmsh
    g = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mignon3dB.json")))
    p = str(tmp_path / "mignon3dB.msh")
    _write_gmsh(p, g)
    mesh = mg.Mesh.load_gmsh(p, order=1)
    sel, _ = mesh.triangles(geo_ids=[2])
    b = mg.MatrixBuilder(mesh)
    lg = mg.LagrangeBuilder(b, tris=sel, test_order=0)
    got = lg.assemble(quad=3).cpu().numpy()
    xyz, conn = mesh.geometry()
    lam, rp, ci, ref, _, _ = orc.lagrange(1, 3, xyz, conn, mesh.elem_dofs(), b.ndof, tris=sel, test_order=0)
    assert lg.n_multipliers == 4 and row_scaled_err(rp, ref, got) <= 1e-12


@pytest.mark.parametrize("order", [1, 2])
def test_saddle_with_mtm_and_mmt_matches_oracle(order):
    """setMTM and setMMT together: K + eI + a B^T B and eI + b B B^T."""
    m, mesh, b, _, _ = _setup(4 if order == 1 else 3, order, 30)
    lg = mg.LagrangeBuilder(b, lam_diag=True, mtm=True, mmt=True)
    K = b.assemble("stiff_const", quad=4)
    B = lg.assemble(quad=3)
    S = lg.saddle(K, B, eye_field=0.5, eye_lam=-0.25, mtm_scale=3.0, mmt_scale=-2.0)
    dofs, rp, ci, kref = orc.full_operator("stiff_const", order, 4, m.xyz, m.conn)
    _, brp, bci, bref, _, _ = orc.lagrange(order, 3, m.xyz, m.conn, dofs, b.ndof)
    srp, sci, sref = orc.saddle(rp, ci, kref, brp, bci, bref, b.ndof, lam_diag=True, eye_field=0.5, eye_lam=-0.25,
                                with_mtm=True, mtm_scale=3.0, with_mmt=True, mmt_scale=-2.0)
    (_, _), (gsrp, gsci) = lg.pattern()
    assert np.array_equal(gsrp, srp) and np.array_equal(gsci, sci)
    assert row_scaled_err(srp, sref, S.cpu().numpy()) <= 1e-12


def test_p2_multipliers_on_first_numbered_mesh():
    m = meshgen.kuhn_cube(3, jitter=0.2, seed=31, permute=True)
    mesh = mg.Mesh(m.xyz, m.conn, order=2, edge_rule="first")
    b = mg.MatrixBuilder(mesh)
    lg = mg.LagrangeBuilder(b, test_order=2)
    got = lg.assemble(quad=6).cpu().numpy()
    lam, rp, ci, ref, _, _ = orc.lagrange(2, 6, m.xyz, m.conn, mesh.elem_dofs(), b.ndof, test_order=2,
                                          edge_rule="first")
    (brp, bci), _ = lg.pattern()
    assert np.array_equal(brp, rp) and np.array_equal(bci, ci)
    assert row_scaled_err(rp, ref, got) <= 1e-12
