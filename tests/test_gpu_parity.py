"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle.

Tolerances: CSR pattern and dof numbering bit-exact; FP64 values row-scaled
|a-b| <= 1e-12 max(|a|, max_j |A_row,j|); FP32 values row-scaled 2e-6;
solutions against the FP64 oracle solution at the stated tolerances."""
import numpy as np
import pytest

import morganapublic_gb300 as mg
import oracle as orc
from morganapublic_gb300 import meshgen
from helpers import (disjoint_tets, emulate_block_map, emulate_slot_map, expected_block_map, expected_slot_map,
                     row_scaled_err, star_mesh)

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

F64_TOL = 1e-12
F32_TOL = 2e-6


def _case(n, jitter, seed, permute, sigma):
    m = meshgen.kuhn_cube(n, jitter=jitter, seed=seed, permute=permute)
    kappa = meshgen.lognormal(len(m.conn), sigma, seed + 100) if sigma > 0 else np.ones(len(m.conn))
    return m, kappa


@pytest.mark.parametrize("op", ["stiff_kappa", "stiff_const", "mass", "mass_coeff"])
@pytest.mark.parametrize("quad", [1, 4, 15, 64])
def test_p1_assembly_f64(op, quad):
    # the 64-point card (weights summing to 1/6 - 5e-11) with a constant coefficient
    # puts many entries just below a power of two: the double-word to double
    # conversion must step into the binade below with its ulp
    m, kappa = _case(6, 0.2, 1, True, 1.0)
    mesh = mg.Mesh(m.xyz, m.conn, order=1)
    b = mg.MatrixBuilder(mesh)
    dofs, rp, ci, ref = orc.full_operator(op, 1, quad, m.xyz, m.conn, coeff=kappa, c=2.5)
    vals = b.assemble(op, coeff=kappa, c=2.5, quad=quad, prec="f64").cpu().numpy()
    rph, cih = b.pattern()
    assert np.array_equal(rph, rp) and np.array_equal(cih, ci)
    assert row_scaled_err(rp, ref, vals) <= F64_TOL


@pytest.mark.parametrize("op", ["stiff_kappa", "mass"])
def test_p1_assembly_f32(op):
    m, kappa = _case(6, 0.25, 3, True, 1.5)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    _, rp, ci, ref = orc.full_operator(op, 1, 4, m.xyz, m.conn, coeff=kappa)
    vals = b.assemble(op, coeff=kappa, quad=4, prec="f32").cpu().numpy()
    assert vals.dtype == np.float32
    assert row_scaled_err(rp, ref, vals) <= F32_TOL


@pytest.mark.parametrize("op", ["stiff_kappa", "mass", "stiff_const", "mass_coeff"])
@pytest.mark.parametrize("rule", ["lex", "first"])
def test_p2_assembly_f64(op, rule):
    m, kappa = _case(3, 0.2, 2, True, 0.5)
    mesh = mg.Mesh(m.xyz, m.conn, order=2, edge_rule=rule)
    b = mg.MatrixBuilder(mesh)
    dofs, rp, ci, ref = orc.full_operator(op, 2, 15, m.xyz, m.conn, coeff=kappa, c=0.75, edge_rule=rule)
    assert np.array_equal(mesh.elem_dofs(), dofs)
    for quad in (15, 11):  # Keast 11 is exact for these degree <= 4 integrands on affine tets
        vals = b.assemble(op, coeff=kappa, c=0.75, quad=quad, prec="f64").cpu().numpy()
        assert row_scaled_err(rp, ref, vals) <= F64_TOL, quad
    # the under-integrating cards, and the 64-point card (its 10-digit constants
    # move the values by ~1e-9), against the oracle with the same card
    for quad in (1, 4, 64):
        _, _, _, ref_q = orc.full_operator(op, 2, quad, m.xyz, m.conn, coeff=kappa, c=0.75, edge_rule=rule)
        vals = b.assemble(op, coeff=kappa, c=0.75, quad=quad, prec="f64").cpu().numpy()
        assert row_scaled_err(rp, ref_q, vals) <= F64_TOL, quad


def test_p2_assembly_f32():
    m, kappa = _case(3, 0.2, 2, True, 0.5)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=2))
    _, rp, ci, ref = orc.full_operator("stiff_kappa", 2, 15, m.xyz, m.conn, coeff=kappa)
    vals = b.assemble("stiff_kappa", coeff=kappa, quad=11, prec="f32").cpu().numpy()
    assert row_scaled_err(rp, ref, vals) <= 2 * F32_TOL


@pytest.mark.parametrize("case", ["jitter_s5", "jitter_s6", "jitter_s7", "sliver_1e-2", "sliver_1e-3", "sliver_1e-4"])
def test_near_degenerate_elements(case):
    """Elements whose determinant cancels in its cofactor expansion (Kuhn cubes
    jittered by 0.49 h, cancellation up to ~230; single slivers of relative height
    1e-2..1e-4 in a rotated plane): those elements take the FP64 geometry path, so
    the double-word values keep FP64 parity and the FP32 values stay accurate."""
    if case.startswith("jitter"):
        seed = int(case[-1])
        m = meshgen.kuhn_cube(8, jitter=0.49, seed=seed, permute=True)
        xyz, conn, kappa = m.xyz, m.conn, meshgen.lognormal(len(m.conn), 1.0, seed)
    else:
        eps = float(case.split("_")[1])
        Q, _ = np.linalg.qr(np.random.default_rng(1).standard_normal((3, 3)))
        base = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.3, 0.3, eps]], dtype=np.float64)
        xyz = 0.37 + 0.1 * base @ Q.T
        d = np.linalg.det(np.stack([xyz[k] - xyz[0] for k in (1, 2, 3)], axis=1))
        conn = np.array([[0, 1, 2, 3]] if d > 0 else [[0, 2, 1, 3]], dtype=np.int32)
        kappa = np.ones(1)
    b = mg.MatrixBuilder(mg.Mesh(xyz, conn, order=1))
    _, rp, ci, ref = orc.full_operator("stiff_kappa", 1, 4, xyz, conn, coeff=kappa)
    v64 = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64").cpu().numpy()
    v32 = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f32").cpu().numpy()
    assert row_scaled_err(rp, ref, v64) <= F64_TOL
    assert row_scaled_err(rp, ref, v32) <= 1e-5


def test_assembly_deterministic_and_host_entry():
    m, kappa = _case(8, 0.25, 3, True, 1.5)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    v1 = b.assemble("stiff_kappa", coeff=kappa, prec="f64")
    v2 = b.assemble("stiff_kappa", coeff=kappa, prec="f64")
    assert torch.equal(v1, v2)
    crs = b.build_crs("stiff_kappa", coeff=kappa, prec="f64")
    assert np.array_equal(crs.values, v1.cpu().numpy())


def test_config1_laplace_and_mass_16():
    """The reference's CPU-runnable case: P1 16^3 Kuhn cube, kappa = 1, 4-point rule."""
    m = meshgen.kuhn_cube(16)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    assert (b.ndof, b.nnz) == (4913, 66961)
    for op in ("stiff_kappa", "mass"):
        _, rp, ci, ref = orc.full_operator(op, 1, 4, m.xyz, m.conn, coeff=np.ones(len(m.conn)))
        vals = b.assemble(op, coeff=np.ones(len(m.conn)), quad=4, prec="f64").cpu().numpy()
        assert row_scaled_err(rp, ref, vals) <= F64_TOL


def test_spmv_matches_oracle():
    m, kappa = _case(8, 0.2, 1, True, 1.0)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    _, rp, ci, ref = orc.full_operator("stiff_kappa", 1, 4, m.xyz, m.conn, coeff=kappa)
    x = np.random.default_rng(0).uniform(-1, 1, b.ndof)
    y_ref = orc.spmv(rp, ci, ref, x)
    vals = b.assemble("stiff_kappa", coeff=kappa, prec="f64")
    y = b.apply(vals, torch.from_numpy(x).cuda()).cpu().numpy()
    scale = np.abs(ref).max() * np.abs(x).max()
    assert np.max(np.abs(y - y_ref)) <= 1e-13 * scale * 27
    v32 = b.assemble("stiff_kappa", coeff=kappa, prec="f32")
    y32 = b.apply(v32, torch.from_numpy(x.astype(np.float32)).cuda()).cpu().numpy()
    assert np.max(np.abs(y32 - y_ref)) <= 1e-5 * scale


def _dirichlet_system(n, order, sigma, seed):
    m, kappa = _case(n, 0.2, seed, True, sigma)
    mesh = mg.Mesh(m.xyz, m.conn, order=order)
    b = mg.MatrixBuilder(mesh)
    quad = 4 if order == 1 else 15
    dofs, rp, ci, K = orc.full_operator("stiff_kappa", order, quad, m.xyz, m.conn, coeff=kappa)
    mask = m.boundary if order == 1 else meshgen.p2_boundary(m.boundary, mesh.edges()[0])
    rhs = orc.assemble_rhs(order, quad, m.xyz, m.conn, dofs, b.ndof)
    return m, kappa, mesh, b, dofs, rp, ci, K, mask, rhs, quad


def test_rhs_and_dirichlet_match_oracle():
    m, kappa, mesh, b, dofs, rp, ci, K, mask, rhs, quad = _dirichlet_system(6, 1, 1.0, 4)
    bg = b.build_vector(quad=quad).cpu().numpy()
    assert np.max(np.abs(bg - rhs)) <= 1e-15 * 30
    f = np.sin(np.pi * m.xyz[:, 0])
    rhs_f = orc.assemble_rhs(1, quad, m.xyz, m.conn, dofs, b.ndof, field=f, elem_scale=kappa)
    bf = b.build_vector(field=f, elem_scale=kappa, quad=quad).cpu().numpy()
    assert np.max(np.abs(bf - rhs_f)) <= 1e-13 * np.abs(rhs_f).max()
    Kd = K.copy()
    rd = rhs.copy()
    orc.apply_dirichlet(rp, ci, mask, Kd, rd)
    v = b.assemble("stiff_kappa", coeff=kappa, quad=quad)
    bt = torch.from_numpy(rhs).cuda()
    b.apply_dirichlet(v, torch.from_numpy(mask), bt)
    assert row_scaled_err(rp, Kd, v.cpu().numpy()) <= F64_TOL
    assert np.array_equal(bt.cpu().numpy(), rd)


@pytest.mark.parametrize("order", [1, 2])
def test_cg_and_refined_vs_oracle(order):
    m, kappa, mesh, b, dofs, rp, ci, K, mask, rhs, quad = _dirichlet_system(6 if order == 1 else 4, order, 1.0, 5)
    orc.apply_dirichlet(rp, ci, mask, K, rhs)
    x_ref, it_ref, rr_ref, rc = orc.cg(rp, ci, K, rhs, rtol=1e-13)
    assert rc == 0
    v64 = b.assemble("stiff_kappa", coeff=kappa, quad=quad, prec="f64")
    v32 = b.assemble("stiff_kappa", coeff=kappa, quad=quad, prec="f32")
    mk = torch.from_numpy(mask)
    bt = torch.from_numpy(rhs).cuda()
    b.apply_dirichlet(v64, mk)
    b.apply_dirichlet(v32, mk)
    x, info = b.cg(v64, bt, rtol=1e-10, precond="jacobi")
    assert info.converged and info.rel_residual <= 1e-10
    err = np.linalg.norm(x.cpu().numpy() - x_ref) / np.linalg.norm(x_ref)
    assert err <= 1e-8
    xr, infor = b.cg_refined(v64, v32, bt, rtol=1e-10, inner_rtol=1e-4)
    assert infor.converged and infor.rel_residual <= 1e-10 and infor.outer_iterations >= 1
    err_r = np.linalg.norm(xr.cpu().numpy() - x_ref) / np.linalg.norm(x_ref)
    assert err_r <= 1e-8
    # the FP64 residual of the refined solution, recomputed by the oracle
    r = rhs - orc.spmv(rp, ci, K, xr.cpu().numpy())
    assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(rhs)


def test_manufactured_p2_mixed_vs_fp64_against_oracle():
    """The P2 mixed-precision workload in small: rhs = A u_I for the P2 interpolant
    u_I of sin(pi x) sin(pi y) sin(pi z) (zero on the boundary, Dirichlet rows
    eliminated), so u_I is the exact discrete solution.  FP64 CG and the
    reliable-update mixed-precision CG (default trigger) both reach 1e-10; their
    solutions are compared with the oracle's FP64 CG solution and with u_I, and
    the FP32 Krylov sequence is not restarted (iterations close to FP64's)."""
    n, quad = 5, 15
    m, kappa = _case(n, 0.0, 11, False, 0.5)
    mesh = mg.Mesh(m.xyz, m.conn, order=2)
    b = mg.MatrixBuilder(mesh)
    dofs, rp, ci, K = orc.full_operator("stiff_kappa", 2, quad, m.xyz, m.conn, coeff=kappa)
    en = mesh.edges()[0]
    mask = meshgen.p2_boundary(m.boundary, en)
    X = np.concatenate([m.xyz, 0.5 * (m.xyz[en[:, 0]] + m.xyz[en[:, 1]])])
    uI = np.sin(np.pi * X[:, 0]) * np.sin(np.pi * X[:, 1]) * np.sin(np.pi * X[:, 2])
    uI[mask] = 0.0
    orc.apply_dirichlet(rp, ci, mask, K)
    rhs = orc.spmv(rp, ci, K, uI)
    x_ref, it_ref, _, rc = orc.cg(rp, ci, K, rhs, rtol=1e-13)
    assert rc == 0
    v64 = b.assemble("stiff_kappa", coeff=kappa, quad=quad, prec="f64")
    v32 = b.assemble("stiff_kappa", coeff=kappa, quad=quad, prec="f32")
    mk = torch.from_numpy(mask)
    b.apply_dirichlet(v64, mk)
    b.apply_dirichlet(v32, mk)
    bt = b.apply(v64, torch.from_numpy(uI).cuda())
    assert np.max(np.abs(bt.cpu().numpy() - rhs)) <= 1e-12 * np.abs(rhs).max()
    x, info = b.cg(v64, bt, rtol=1e-10)
    xr, infor = b.cg_refined(v64, v32, bt, rtol=1e-10)
    assert info.converged and infor.converged and infor.rel_residual <= 1e-10
    for sol in (x.cpu().numpy(), xr.cpu().numpy()):
        assert np.linalg.norm(sol - x_ref) / np.linalg.norm(x_ref) <= 1e-8
        assert np.linalg.norm(sol - uI) / np.linalg.norm(uI) <= 1e-8
    assert infor.iterations <= 1.5 * info.iterations + 20


def test_unreferenced_nodes_give_empty_rows():
    """Nodes no element references (common in Gmsh files) own empty CSR rows.
    3000 of them scattered through a 4^3 mesh put more than 2048 rows (the
    per-block row cap) into a block of few entries; pattern, values and SpMV
    still match the oracle."""
    m, kappa = _case(4, 0.2, 9, True, 1.0)
    extra = np.random.default_rng(9).uniform(0.0, 1.0, (3000, 3))
    xyz = np.concatenate([m.xyz, extra])
    b = mg.MatrixBuilder(mg.Mesh(xyz, m.conn, order=1))
    assert b.ndof == len(xyz)
    dofs, rp, ci, ref = orc.full_operator("stiff_kappa", 1, 4, xyz, m.conn, coeff=kappa)
    rph, cih = b.pattern()
    assert np.array_equal(rph, rp) and np.array_equal(cih, ci)
    assert np.all(np.diff(rp)[len(m.xyz):] == 0)
    v = b.assemble("stiff_kappa", coeff=kappa, quad=4)
    assert row_scaled_err(rp, ref, v.cpu().numpy()) <= F64_TOL
    x = np.random.default_rng(1).uniform(-1, 1, len(xyz))
    y = b.apply(v, torch.from_numpy(x).cuda()).cpu().numpy()
    y_ref = orc.spmv(rp, ci, ref, x)
    assert np.max(np.abs(y - y_ref)) <= 1e-12 * np.abs(y_ref).max()
    f = np.random.default_rng(2).uniform(-1, 1, len(xyz))
    r_ref = orc.assemble_rhs(1, 4, xyz, m.conn, dofs, b.ndof, field=f, elem_scale=kappa)
    r = b.build_vector(field=f, elem_scale=kappa, quad=4).cpu().numpy()
    assert np.all(r[len(m.xyz):] == 0.0)
    assert np.max(np.abs(r - r_ref)) <= 1e-13 * np.abs(r_ref).max()


@pytest.mark.parametrize("case", ["p1", "p2_lex", "p2_first", "extra_nodes", "single", "no_elements", "p1_big",
                                  "p2_big"])
def test_device_pattern_build_matches_host(case):
    """mg_pattern_build_device (CSR pattern from sorted element-coupling keys, the
    Morton element order and the slot map, all on the GPU) gives the host build's
    arrays bit for bit, hence the same values."""
    xyz1 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    if case == "single":
        xyz, conn, order, rule = xyz1, np.array([[0, 1, 2, 3]], dtype=np.int32), 1, "lex"
    elif case == "no_elements":
        xyz, conn, order, rule = xyz1, np.zeros((0, 4), dtype=np.int32), 1, "lex"
    elif case.endswith("big"):
        m = meshgen.kuhn_cube(32 if case == "p1_big" else 12, jitter=0.25, seed=19, permute=True)
        xyz, conn, order, rule = m.xyz, m.conn, 1 if case == "p1_big" else 2, "lex"
    else:
        m = meshgen.kuhn_cube(6 if case.startswith("p1") or case == "extra_nodes" else 4, jitter=0.2, seed=17,
                              permute=True)
        xyz, conn = m.xyz, m.conn
        if case == "extra_nodes":
            xyz = np.concatenate([xyz, np.random.default_rng(3).uniform(0, 1, (500, 3))])
        order = 2 if case.startswith("p2") else 1
        rule = "first" if case == "p2_first" else "lex"
    mesh = mg.Mesh(xyz, conn, order=order, edge_rule=rule)
    host = mg.MatrixBuilder(mesh)
    dev = mg.MatrixBuilder(mesh, pattern_on_device=True)
    assert (dev.ndof, dev.nnz) == (host.ndof, host.nnz)
    rp_h, ci_h = host.pattern()
    rp_d, ci_d = dev.pattern()
    assert np.array_equal(rp_h, rp_d) and np.array_equal(ci_h, ci_d)
    if order == 1:
        sh, sd = host.export_block_map(), dev.export_block_map()
        fields = ("n_upper", "n_contrib", "n_blocks", "n_groups", "n_src", "n_runs", "n_shared", "n_shared_groups",
                  "n_partial", "n_elem", "nunique", "elems_per_block")
    else:
        sh, sd = host.export_slot_map(), dev.export_slot_map()
        fields = ("n_upper", "n_groups", "n_diag", "n_contrib", "n_src", "n_elem", "nunique", "elem_major",
                  "rows_per_block")
    for f in fields:
        assert getattr(sh["info"], f) == getattr(sd["info"], f), f
    for k in sh:
        if k != "info":
            assert np.array_equal(np.asarray(sh[k]), np.asarray(sd[k])), k
    if len(conn):
        kappa = meshgen.lognormal(len(conn), 1.0, 5)
        vh = host.assemble("stiff_kappa", coeff=kappa, quad=4).cpu().numpy()
        vd = dev.assemble("stiff_kappa", coeff=kappa, quad=4).cpu().numpy()
        assert np.array_equal(vh.view(np.int64), vd.view(np.int64))


@pytest.mark.parametrize("rule", ["lex", "first"])
@pytest.mark.parametrize("n,permute", [(1, False), (3, True), (7, True)])
def test_device_edges_match_host(rule, n, permute):
    """mg_mesh_create_device (P2 edges enumerated on the GPU) gives the host's edge
    table, element-to-edge table and dof map bit for bit, for both numbering rules."""
    m = meshgen.kuhn_cube(n, jitter=0.2 if n > 1 else 0.0, seed=23, permute=permute)
    host = mg.Mesh(m.xyz, m.conn, order=2, edge_rule=rule)
    dev = mg.Mesh(m.xyz, m.conn, order=2, edge_rule=rule, edges_on_device=True)
    en_h, ee_h = host.edges()
    en_d, ee_d = dev.edges()
    assert np.array_equal(en_h, en_d) and np.array_equal(ee_h, ee_d)
    assert np.array_equal(host.elem_dofs(), dev.elem_dofs())
    if n == 3:
        en_o, ee_o = orc.edges(len(m.xyz), m.conn, rule)
        assert np.array_equal(en_d, en_o) and np.array_equal(ee_d, ee_o)
    # P1 meshes and meshes without elements take the same entry point
    assert mg.Mesh(m.xyz, m.conn, order=1, edges_on_device=True).ndof == len(m.xyz)
    assert mg.Mesh(m.xyz, np.zeros((0, 4), dtype=np.int32), order=2, edges_on_device=True).ndof == len(m.xyz)


def test_nonfinite_coefficient_is_reported():
    """A NaN or Inf in the per-element coefficient is an error returned through
    the C ABI (mg_plan_status; the host-buffer call checks it itself); a clean
    assembly afterwards reports nothing."""
    m, kappa = _case(3, 0.2, 12, True, 1.0)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    for bad in (np.nan, np.inf):
        k = kappa.copy()
        k[len(k) // 2] = bad
        b.assemble("stiff_kappa", coeff=torch.from_numpy(k).cuda(), quad=4)
        with pytest.raises(mg.MorganaError) as e:
            b.status()
        assert e.value.status == mg.MG_ERR_INVALID_ARG
        with pytest.raises(mg.MorganaError) as e:
            b.build_crs("stiff_kappa", coeff=k, quad=4)
        assert e.value.status == mg.MG_ERR_INVALID_ARG
    b.assemble("stiff_kappa", coeff=torch.from_numpy(kappa).cuda(), quad=4)
    b.status()


def test_concurrent_plans_on_host_threads():
    """One handle per host thread: two threads assemble and apply plans of
    different sizes (different shared-memory needs) on their own streams at the
    same time; every result equals the one computed alone, bit for bit."""
    import threading
    cases = []
    for n, order in ((5, 1), (3, 2)):
        m, kappa = _case(n, 0.2, 20 + n, True, 1.0)
        b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=order))
        kap = torch.from_numpy(kappa).cuda()
        x = torch.from_numpy(np.random.default_rng(n).uniform(-1, 1, b.ndof)).cuda()
        q = 4 if order == 1 else 15
        ref_v = b.assemble("stiff_kappa", coeff=kap, quad=q)
        ref_y = b.apply(ref_v, x)
        torch.cuda.synchronize()
        cases.append((b, kap, x, q, ref_v, ref_y))
    errors = []

    def work(case):
        b, kap, x, q, ref_v, ref_y = case
        st = torch.cuda.Stream()
        try:
            for _ in range(5):
                v = b.assemble("stiff_kappa", coeff=kap, quad=q, stream=st)
                y = b.apply(v, x, stream=st)
                st.synchronize()
                if not (torch.equal(v, ref_v) and torch.equal(y, ref_y)):
                    errors.append("mismatch")
            b.status()
        except Exception as ex:  # reported to the main thread
            errors.append(repr(ex))

    ts = [threading.Thread(target=work, args=(c,)) for c in cases]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors


def test_cg_deterministic_and_maxit_status():
    m, kappa, mesh, b, dofs, rp, ci, K, mask, rhs, quad = _dirichlet_system(5, 1, 1.0, 6)
    v = b.assemble("stiff_kappa", coeff=kappa, quad=quad)
    bt = torch.from_numpy(rhs).cuda()
    b.apply_dirichlet(v, torch.from_numpy(mask), bt)
    x1, i1 = b.cg(v, bt, rtol=1e-10)
    x2, i2 = b.cg(v, bt, rtol=1e-10)
    assert torch.equal(x1, x2) and i1.iterations == i2.iterations
    x3, i3 = b.cg(v, bt, rtol=1e-14, maxit=3, raise_on_fail=False)
    assert not i3.converged and i3.iterations == 3
    with pytest.raises(mg.MorganaError) as e:
        b.cg(v, bt, rtol=1e-14, maxit=3)
    assert e.value.status == mg.MG_ERR_NOT_CONVERGED


@pytest.mark.parametrize("op", ["stiff_kappa", "mass_coeff"])
def test_p2_native_f64_assembly(op):
    """MG_F64_NATIVE (native FP64 element arithmetic) on P2 against the oracle, and
    against the double-word MG_F64 values."""
    m, kappa = _case(3, 0.2, 13, True, 1.0)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=2))
    _, rp, ci, ref = orc.full_operator(op, 2, 15, m.xyz, m.conn, coeff=kappa)
    nat = b.assemble(op, coeff=kappa, quad=15, prec="f64_native").cpu().numpy()
    dw = b.assemble(op, coeff=kappa, quad=15, prec="f64").cpu().numpy()
    b.status()
    assert row_scaled_err(rp, ref, nat) <= F64_TOL
    assert row_scaled_err(rp, nat, dw) <= F64_TOL


@pytest.mark.parametrize("order,quad", [(1, 1), (1, 4), (1, 15), (1, 64), (2, 4), (2, 11), (2, 15), (2, 64)])
@pytest.mark.parametrize("scale", [1e-30, 1.0, 1e30])
def test_load_vector_against_oracle(order, quad, scale):
    """mg_assemble_rhs (element vectors + fixed-order per-dof sums) against the
    oracle's vector builder: with and without a nodal field and an element
    scale, at coefficient / field scales far from 1, FP64 within 1e-13 of
    max |b|; two calls give the same bits."""
    n = 5 if order == 1 else 3
    m, kappa = _case(n, 0.2, 21, True, 1.0)
    mesh = mg.Mesh(m.xyz, m.conn, order=order)
    b = mg.MatrixBuilder(mesh)
    dofs = mesh.elem_dofs()
    X = m.xyz if order == 1 else np.concatenate([m.xyz, 0.5 * (m.xyz[mesh.edges()[0][:, 0]] + m.xyz[mesh.edges()[0][:, 1]])])
    f = (np.sin(3.0 * X[:, 0]) + X[:, 1] * X[:, 2] - 0.3) * scale
    f[::9] = 0.0
    s = kappa * scale
    for field, es in ((None, None), (f, None), (None, s), (f, s)):
        # the oracle holds the reference's cards; Keast 11 is exact to degree 4, like card 15 here
        ref = orc.assemble_rhs(order, 15 if quad == 11 else quad, m.xyz, m.conn, dofs, b.ndof, field=field,
                               elem_scale=es)
        got = b.build_vector(field=field, elem_scale=es, quad=quad).cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.max(np.abs(got - ref)) <= 1e-13 * np.abs(ref).max()
        again = b.build_vector(field=field, elem_scale=es, quad=quad).cpu().numpy()
        assert np.array_equal(got.view(np.int64), again.view(np.int64))


@pytest.mark.parametrize("order", [1, 2])
def test_adjoint_gradient(order):
    """dJ/dkappa_e from the adjoint kernel against the oracle gradient and
    central finite differences of J(kappa) = 1/2 ||u(kappa) - u_t||^2."""
    n = 4 if order == 1 else 3
    m, kappa, mesh, b, dofs, rp, ci, K, mask, rhs, quad = _dirichlet_system(n, order, 0.5, 7)
    ut = np.random.default_rng(1).uniform(0, 0.05, b.ndof) * (~mask)
    mk = torch.from_numpy(mask)

    def solve(kap):
        v = b.assemble("stiff_kappa", coeff=kap, quad=quad)
        bt = torch.from_numpy(rhs).cuda()
        b.apply_dirichlet(v, mk, bt)
        x, _ = b.cg(v, bt, rtol=1e-13, maxit=20000)
        return v, x

    v, u = solve(kappa)
    res = u - torch.from_numpy(ut).cuda()
    lam, _ = b.cg(v, res.clone(), rtol=1e-13, maxit=20000)
    g = b.adjoint_grad(u, lam, quad=quad).cpu().numpy()
    g_ref = orc.adjoint_grad(order, quad, m.xyz, m.conn, dofs, u.cpu().numpy(), lam.cpu().numpy())
    assert np.max(np.abs(g - g_ref)) <= 1e-12 * np.abs(g_ref).max()
    J = lambda uu: 0.5 * float(((uu - torch.from_numpy(ut).cuda()) ** 2).sum())
    for e in np.random.default_rng(3).choice(len(kappa), 8, replace=False):
        h = 1e-5 * kappa[e]
        kp, km = kappa.copy(), kappa.copy()
        kp[e] += h
        km[e] -= h
        fd = (J(solve(kp)[1]) - J(solve(km)[1])) / (2 * h)
        assert abs(fd - g[e]) <= 1e-5 * np.abs(g).max() + 1e-6 * abs(fd)


@pytest.mark.parametrize("scale", [1e-30, 1e-24, 1e-12, 1.0, 1e12, 1e24, 1e36])
def test_extreme_scales_assembly_and_adjoint(scale):
    """Coefficients, u and lambda far from 1.  The double-word (MG_F64) assembly
    keeps FP64 parity while element scales stay within 2^-96 .. 2^112 and reports
    MG_ERR_UNSUPPORTED through mg_plan_status outside it; MG_F64_NATIVE covers
    the whole range.  The adjoint rescales each element's differences by powers
    of two, so it keeps parity at every scale (conversions inside and outside
    the integer-conversion range, zero coefficients and zero values included)."""
    m, kappa = _case(4, 0.2, 11, True, 1.0)
    kappa = kappa * scale
    kappa[::7] = 0.0
    mesh = mg.Mesh(m.xyz, m.conn, order=1)
    b = mg.MatrixBuilder(mesh)
    dofs, rp, ci, ref = orc.full_operator("stiff_kappa", 1, 4, m.xyz, m.conn, coeff=kappa)
    kt = torch.from_numpy(kappa).cuda()
    in_range = 1e-24 <= scale <= 1e24
    vals = b.assemble("stiff_kappa", coeff=kt, quad=4, prec="f64").cpu().numpy()
    if in_range:
        b.status()
        assert row_scaled_err(rp, ref, vals) <= F64_TOL
    else:
        with pytest.raises(mg.MorganaError) as e:
            b.status()
        assert e.value.status == mg.MG_ERR_UNSUPPORTED
    nat = b.assemble("stiff_kappa", coeff=kt, quad=4, prec="f64_native").cpu().numpy()
    b.status()
    assert nat.dtype == np.float64
    assert row_scaled_err(rp, ref, nat) <= F64_TOL
    rng = np.random.default_rng(5)
    u = rng.uniform(-1, 1, b.ndof) * scale
    lam = rng.uniform(-1, 1, b.ndof) * scale
    u[::5] = 0.0
    g = b.adjoint_grad(torch.from_numpy(u).cuda(), torch.from_numpy(lam).cuda(), quad=4).cpu().numpy()
    g_ref = orc.adjoint_grad(1, 4, m.xyz, m.conn, dofs, u, lam)
    assert np.all(np.isfinite(g))
    assert np.max(np.abs(g - g_ref)) <= 1e-12 * np.abs(g_ref).max()


def test_gmsh_loaded_mesh_assembles(tmp_path):
    m, kappa = _case(4, 0.2, 8, True, 1.0)
    p = str(tmp_path / "c.msh")
    meshgen.write_gmsh(p, m.xyz, m.conn)
    b = mg.MatrixBuilder(mg.Mesh.load_gmsh(p, order=1))
    _, rp, ci, ref = orc.full_operator("stiff_kappa", 1, 4, m.xyz, m.conn, coeff=kappa)
    vals = b.assemble("stiff_kappa", coeff=kappa).cpu().numpy()
    assert row_scaled_err(rp, ref, vals) <= F64_TOL


@pytest.mark.parametrize("order,rule", [(1, "lex"), (2, "lex"), (2, "first")])
def test_reference_fixture_mignon3dC(order, rule, tmp_path):
    """The reference's own unit-test cases on its mignon3dC.msh mesh (7 nodes,
    8 tets; tests/morganaIntegrator/integratorOEL3d_STDTest1.cpp: opEL3dA with
    kappa = 12, tests/morganaFiniteElements/localMatrixEL3dTest1.cpp: kappa = 1):
    the mesh from its fixture (tests/golden/mignon3dC.json) written back as a Gmsh 2
    file, loaded through the Gmsh reader and assembled on the GPU with every
    quadrature card and operator, against the oracle."""
    import json
    import os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "mignon3dC.json")))
    xyz = np.array(g["nodes"], dtype=np.float64)
    conn = np.array(g["tets_1based"], dtype=np.int32) - 1
    path = str(tmp_path / "mignon3dC.msh")
    meshgen.write_gmsh(path, xyz, conn)
    mesh = mg.Mesh.load_gmsh(path, order=order, edge_rule=rule)
    gx, gc = mesh.geometry()
    assert np.array_equal(gx, xyz) and np.array_equal(gc, conn)
    b = mg.MatrixBuilder(mesh)
    for op, coef in (("stiff_kappa", 12.0), ("stiff_kappa", 1.0), ("stiff_const", 12.0), ("mass", 1.0),
                     ("mass_coeff", 12.0)):
        kappa = np.full(len(conn), coef)
        for quad in (1, 4, 15, 64):
            dofs, rp, ci, ref = orc.full_operator(op, order, quad, xyz, conn, coeff=kappa, c=coef, edge_rule=rule)
            assert np.array_equal(mesh.elem_dofs(), dofs)
            rph, cih = b.pattern()
            assert np.array_equal(rph, rp) and np.array_equal(cih, ci)
            vals = b.assemble(op, coeff=kappa, c=coef, quad=quad, prec="f64").cpu().numpy()
            assert row_scaled_err(rp, ref, vals) <= F64_TOL, (op, coef, quad)


def test_single_tet_and_empty():
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    b = mg.MatrixBuilder(mg.Mesh(xyz, np.array([[0, 1, 2, 3]], dtype=np.int32)))
    K = b.assemble("stiff_kappa", coeff=np.ones(1)).cpu().numpy().reshape(4, 4)
    assert np.allclose(K, np.array([[3, -1, -1, -1], [-1, 1, 0, 0], [-1, 0, 1, 0], [-1, 0, 0, 1]]) / 6.0,
                       atol=1e-15)
    # load vector of the reference tet: each vertex gets volume / 4
    f = b.build_vector(quad=4).cpu().numpy()
    assert np.allclose(f, np.full(4, 1.0 / 24.0), rtol=1e-15, atol=0)
    # u = x, lambda = y: grad = -(grad lambda . grad u) vol = 0; u = lambda = x: -vol
    g = b.adjoint_grad(torch.from_numpy(xyz[:, 0].copy()).cuda(), torch.from_numpy(xyz[:, 0].copy()).cuda(),
                       quad=4).cpu().numpy()
    assert abs(g[0] + 1.0 / 6.0) <= 1e-15
    # a mesh of nodes without elements: empty pattern, zero load vector, empty gradient
    e = mg.MatrixBuilder(mg.Mesh(xyz, np.zeros((0, 4), dtype=np.int32)))
    assert e.assemble("mass").numel() == 0
    assert np.all(e.build_vector(quad=4).cpu().numpy() == 0.0)
    assert e.adjoint_grad(torch.zeros(4, dtype=torch.float64, device="cuda"),
                          torch.zeros(4, dtype=torch.float64, device="cuda")).numel() == 0


def test_invalid_arguments_fail_loudly():
    m, kappa = _case(2, 0.0, 1, False, 0.0)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn))
    with pytest.raises(mg.MorganaError) as e:
        b.assemble("stiff_kappa", coeff=None)
    assert e.value.status == mg.MG_ERR_INVALID_ARG
    with pytest.raises(mg.MorganaError):
        b.assemble("mass", quad=7)


# ---------------------------------------------------------------------------
# Against the reference's own code (tests/golden/ref_elements.npz: element
# matrices computed by the reference's compiled quadrature cards, basis
# polynomials, affine map and tensor3d inverse; the 8 tets of its mignon3dC test
# mesh with kappa 12, and 8 jittered tets).  The tets are given disjoint nodes,
# so each element matrix is its own block of the assembled CSR matrix.
REF_QUAD = {1: 1, 2: 4, 3: 15, 4: 64}


def _ref_disjoint():
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_elements.npz"))
    xyz = d["xyz"].reshape(-1, 3).copy()
    conn = np.arange(len(xyz), dtype=np.int32).reshape(-1, 4)
    return d, xyz, conn


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("op", ["stiff_kappa", "stiff_const", "mass", "mass_coeff"])
def test_values_against_reference_code(op, order):
    d, xyz, conn = _ref_disjoint()
    kappa, c = d["kappa"], float(d["c"])
    mesh = mg.Mesh(xyz, conn, order=order)
    b = mg.MatrixBuilder(mesh)
    dofs = mesh.elem_dofs()
    rp, ci = b.pattern()
    nb = dofs.shape[1]
    for prec, quad in REF_QUAD.items():
        ref_mats = d[f"m_{op}_{order}_{prec}"]
        # the CSR matrix the reference's buildEpetraCrs makes of these element blocks
        ref = np.zeros(b.nnz)
        for e in range(len(conn)):
            for i in range(nb):
                for j in range(nb):
                    r, col = dofs[e, j], dofs[e, i]
                    k = rp[r] + np.searchsorted(ci[rp[r]:rp[r + 1]], col)
                    ref[k] += ref_mats[e, i, j]
        v64 = b.assemble(op, coeff=kappa, c=c, quad=quad, prec="f64").cpu().numpy()
        assert row_scaled_err(rp, ref, v64) <= F64_TOL, (prec, row_scaled_err(rp, ref, v64))
        v32 = b.assemble(op, coeff=kappa, c=c, quad=quad, prec="f32").cpu().numpy()
        assert row_scaled_err(rp, ref, v32) <= (F32_TOL if order == 1 else 2 * F32_TOL), prec


def test_adjoint_against_reference_code():
    """dJ/dkappa_e = -lambda_e^T Khat_e u_e with Khat_e the reference's kappa-free
    stiffness (opEL3dF with c = 1), P1 and P2, the 4-point card."""
    d, xyz, conn = _ref_disjoint()
    assert float(d["c"]) == 1.0
    rng = np.random.default_rng(3)
    for order in (1, 2):
        mesh = mg.Mesh(xyz, conn, order=order)
        b = mg.MatrixBuilder(mesh)
        dofs = mesh.elem_dofs()
        u, lam = rng.uniform(-1, 1, b.ndof), rng.uniform(-1, 1, b.ndof)
        khat = d[f"m_stiff_const_{order}_2"]  # [field i, test j]
        g_ref = np.array([-(lam[dofs[e]] @ khat[e].T @ u[dofs[e]]) for e in range(len(conn))])
        g = b.adjoint_grad(torch.from_numpy(u).cuda(), torch.from_numpy(lam).cuda(), quad=4).cpu().numpy()
        assert np.max(np.abs(g - g_ref)) <= 1e-12 * np.abs(g_ref).max(), order


@pytest.mark.parametrize("jitter,seed", [(0.3, 11), (0.35, 12)])
def test_strongly_jittered_mesh_all_entries(jitter, seed):
    """Elements whose vertex-0 gradient is small against the others (|C_max| / |C_0|
    up to ~60 here): the kernel takes that gradient from the coordinates instead of
    the zero row sums, which would cancel; every entry against the oracle."""
    m, kappa = _case(32, jitter, seed, True, 1.5)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    _, rp, ci, ref = orc.full_operator("stiff_kappa", 1, 4, m.xyz, m.conn, coeff=kappa)
    v64 = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64").cpu().numpy()
    b.status()
    assert row_scaled_err(rp, ref, v64) <= F64_TOL
    v32 = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f32").cpu().numpy()
    assert row_scaled_err(rp, ref, v32) <= F32_TOL


@pytest.mark.parametrize("jitter,seed", [(0.25, 13), (0.3, 14)])
def test_strongly_jittered_mesh_p2(jitter, seed):
    """P2 on jittered Kuhn cubes: every entry against the oracle (15-point card on
    both sides)."""
    m, kappa = _case(12, jitter, seed, True, 1.0)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=2))
    _, rp, ci, ref = orc.full_operator("stiff_kappa", 2, 15, m.xyz, m.conn, coeff=kappa)
    v64 = b.assemble("stiff_kappa", coeff=kappa, quad=15, prec="f64").cpu().numpy()
    b.status()
    e64 = row_scaled_err(rp, ref, v64)
    v32 = b.assemble("stiff_kappa", coeff=kappa, quad=15, prec="f32").cpu().numpy()
    e32 = row_scaled_err(rp, ref, v32)
    print(f"P2 12^3 jitter {jitter}: FP64 {e64:.2e}, FP32 {e32:.2e}")
    assert e64 <= F64_TOL and e32 <= 2 * F32_TOL


@pytest.mark.parametrize("n,jitter", [(3, 0.2), (7, 0.25), (12, 0.3)])
def test_block_map_matches_restatement_and_oracle(n, jitter):
    """The device-built block map of a P1 plan equals its numpy restatement bit for
    bit (runs per block, local sources, outputs, partial-sum slots of the shared
    entries), and summing the oracle's element matrices through it gives the
    oracle's CSR values.  12^3 spans 21 element blocks."""
    m = meshgen.kuhn_cube(n, jitter=jitter, seed=8, permute=True)
    kappa = meshgen.lognormal(len(m.conn), 1.0, 6)
    mesh = mg.Mesh(m.xyz, m.conn, order=1)
    b = mg.MatrixBuilder(mesh)
    bm = b.export_block_map()
    rp, ci = b.pattern()
    info = bm["info"]
    assert info.elems_per_block == 512 and info.nunique == 10
    exp = expected_block_map(bm["elem_order"], mesh.elem_dofs(), rp, ci, info.elems_per_block)
    for k in ("bgrp", "goff", "src", "out", "sgoff", "sout"):
        assert np.array_equal(bm[k], exp[k]), k
    assert (info.n_shared, info.n_runs, info.n_upper) == (exp["n_shared"], exp["n_runs"], exp["n_upper"])
    assert info.n_blocks == (len(m.conn) + 511) // 512 and info.n_contrib == 10 * len(m.conn)
    assert (info.n_shared > 0) == (info.n_blocks > 1)
    with pytest.raises(mg.MorganaError):
        b.export_slot_map()  # P1 plans have no two-pass slot map
    dofs, rpo, cio, ref = orc.full_operator("stiff_kappa", 1, 4, m.xyz, m.conn, coeff=kappa)
    mats = [orc.local_matrix("stiff_kappa", 1, 4, m.xyz, m.conn[e], kappa=kappa[e]) for e in range(len(m.conn))]
    got = emulate_block_map(bm, bm["elem_order"], mats, b.nnz)
    assert not np.isnan(got).any()
    assert row_scaled_err(rp, ref, got) <= 1e-14
    v = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64").cpu().numpy()
    assert row_scaled_err(rp, ref, v) <= F64_TOL
    v = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64_native").cpu().numpy()
    assert row_scaled_err(rp, ref, v) <= F64_TOL
    v = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f32").cpu().numpy()
    assert row_scaled_err(rp, ref, v) <= F32_TOL
    b.status()


@pytest.mark.parametrize("case", ["star", "disjoint"])
def test_block_map_beyond_the_shared_memory_stage(case):
    """Blocks whose map does not fit the assembly's shared-memory stage read the rest
    from global memory: a node held by every element (star: a 512-source run, so one
    group pads to 16384 sources, above the 6144 staged) and elements sharing no node
    (disjoint: 160 groups of single-source runs per block, above the 96 group
    offsets staged).  The map equals its restatement and the FP64 / FP32 values the
    oracle's."""
    xyz, conn = star_mesh(700, seed=3) if case == "star" else disjoint_tets(1500, seed=4)
    kappa = meshgen.lognormal(len(conn), 1.0, 21)
    mesh = mg.Mesh(xyz, conn, order=1)
    b = mg.MatrixBuilder(mesh)
    bm = b.export_block_map()
    rp, ci = b.pattern()
    exp = expected_block_map(bm["elem_order"], mesh.elem_dofs(), rp, ci, bm["info"].elems_per_block)
    for k in ("bgrp", "goff", "src", "out", "sgoff", "sout"):
        assert np.array_equal(bm[k], exp[k]), k
    per_block_src = bm["goff"][bm["bgrp"][1:]] - bm["goff"][bm["bgrp"][:-1]]
    per_block_groups = np.diff(bm["bgrp"])
    if case == "star":
        assert per_block_src.max() > 6144
    else:
        assert per_block_groups.max() > 96 and bm["info"].n_shared == 0
    _, rpo, cio, ref = orc.full_operator("stiff_kappa", 1, 4, xyz, conn, coeff=kappa)
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    v64 = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64").cpu().numpy()
    b.status()
    assert row_scaled_err(rp, ref, v64) <= F64_TOL
    v32 = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f32").cpu().numpy()
    assert row_scaled_err(rp, ref, v32) <= F32_TOL
    vn = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64_native").cpu().numpy()
    assert row_scaled_err(rp, ref, vn) <= F64_TOL
    _, _, _, mref = orc.full_operator("mass", 1, 4, xyz, conn)
    vm = b.assemble("mass", quad=4, prec="f64").cpu().numpy()
    assert row_scaled_err(rp, mref, vm) <= F64_TOL


@pytest.mark.parametrize("rule", ["lex", "first"])
def test_high_valence_node_p2(rule):
    """P2 on a star mesh (one vertex starts 700 edges): the edges enumerated on the
    GPU equal the host's, and the assembled P2 operator the oracle's."""
    xyz, conn = star_mesh(700, seed=3)
    kappa = meshgen.lognormal(len(conn), 0.5, 22)
    host = mg.Mesh(xyz, conn, order=2, edge_rule=rule)
    dev = mg.Mesh(xyz, conn, order=2, edge_rule=rule, edges_on_device=True)
    for a, b in zip(host.edges(), dev.edges()):
        assert np.array_equal(a, b)
    assert np.array_equal(host.elem_dofs(), dev.elem_dofs())
    b = mg.MatrixBuilder(dev, pattern_on_device=True)
    _, rp, ci, ref = orc.full_operator("stiff_kappa", 2, 15, xyz, conn, coeff=kappa, edge_rule=rule)
    rph, cih = b.pattern()
    assert np.array_equal(rph, rp) and np.array_equal(cih, ci)
    v = b.assemble("stiff_kappa", coeff=kappa, quad=15, prec="f64").cpu().numpy()
    b.status()
    assert row_scaled_err(rp, ref, v) <= F64_TOL


@pytest.mark.parametrize("order,rule", [(2, "lex"), (2, "first")])
@pytest.mark.parametrize("n,jitter", [(3, 0.2), (4, 0.0), (7, 0.25)])
def test_slot_map_matches_restatement_and_oracle(order, rule, n, jitter):
    """The device-built slot map equals its numpy restatement bit for bit (entries,
    mirrors, sources in ascending Morton position), and summing the oracle's element
    matrices through it gives the oracle's CSR values."""
    m = meshgen.kuhn_cube(n, jitter=jitter, seed=8, permute=True)
    kappa = meshgen.lognormal(len(m.conn), 1.0, 6)
    mesh = mg.Mesh(m.xyz, m.conn, order=order, edge_rule=rule)
    b = mg.MatrixBuilder(mesh)
    sm = b.export_slot_map()
    rp, ci = b.pattern()
    assert sm["info"].rows_per_block == 256
    exp = expected_slot_map(order, sm["elem_order"], mesh.elem_dofs(), rp, ci, sm["info"].rows_per_block)
    for k in ("goff", "uslot", "umirror", "src"):
        assert np.array_equal(sm[k], exp[k]), k
    info = sm["info"]
    assert info.n_diag == exp["n_diag"] == b.ndof and info.elem_major == (order == 1)
    assert info.n_contrib == int(np.sum(exp["src"] != 0xFFFFFFFF)) and info.n_src == len(exp["src"])
    quad = 4 if order == 1 else 15
    dofs, rpo, cio, ref = orc.full_operator("stiff_kappa", order, quad, m.xyz, m.conn, coeff=kappa, edge_rule=rule)
    mats = [orc.local_matrix("stiff_kappa", order, quad, m.xyz, m.conn[e], kappa=kappa[e]) for e in range(len(m.conn))]
    got = emulate_slot_map(sm, order, sm["elem_order"], mats, b.nnz)
    assert not np.isnan(got).any()
    assert row_scaled_err(rp, ref, got) <= 1e-14
