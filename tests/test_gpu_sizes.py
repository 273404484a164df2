"""GPU parity at the benchmark sizes: the meshes bench.py times, checked against
the oracle through the C ABI.

- P1 64^3 (1,572,864 tets; jitter 0.2h, element permutation, lognormal kappa
  sigma 1, seed 1): pattern bit-exact against the oracle's buildEpetraCrs
  restatement, FP64 and FP32 values on every entry, the SpMV against the
  oracle's, and 100 back-to-back SpMVs bitwise identical.
- P2 48^3 (663,552 tets, 912,673 dofs; Keast 11-point rule on the GPU, the
  reference's 15-point card in the oracle -- both exact for these integrands on
  affine tets; lognormal kappa sigma 0.5): pattern bit-exact, values on every
  entry; the FP64 and mixed-precision solves of the oracle's own system
  (rhs = A_oracle u_I for the P2 interpolant u_I, so u_I is its exact discrete
  solution) with each solution's error against it.
- P1 128^3 (12,582,912 tets; jitter 0.25h, permutation, sigma 1.5, seed 3):
  pattern bit-exact on every row, FP64 and FP32 values on 16,384 sampled rows
  (the oracle assembles every element touching one of them, so those rows are
  complete).

Tolerances as in test_gpu_parity: values row-scaled 1e-12 (FP64) / 2e-6 (FP32).
At these sizes the slot map holds up to 1.3e8 sources (P1 128^3) and the
element-matrix array 1 GB, so 32-bit source indices and the gather's grid
run near their largest values of the benchmark."""
import numpy as np
import pytest

import morganapublic_gb300 as mg
import oracle as orc
from morganapublic_gb300 import meshgen
from helpers import row_scaled_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

F64_TOL = 1e-12
F32_TOL = 2e-6


def _rows_err(rowptr, rows, ref, got):
    """row-scaled error over the entries of `rows` only"""
    sl = np.concatenate([np.arange(rowptr[r], rowptr[r + 1]) for r in rows])
    lens = np.diff(rowptr)[rows]
    sub_rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    return row_scaled_err(sub_rp, ref[sl], got[sl])


def test_p1_64cube_full_parity():
    m = meshgen.kuhn_cube(64, jitter=0.2, seed=1, permute=True)
    kappa = meshgen.lognormal(len(m.conn), 1.0, 1)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    assert (b.ndof, b.nnz) == (274625, 4018753)
    dofs = orc.elem_dofs(1, len(m.xyz), m.conn)
    rp, ci = orc.pattern(1, len(m.xyz), dofs)
    rph, cih = b.pattern()
    assert np.array_equal(rph, rp) and np.array_equal(cih, ci)
    ref = orc.assemble("stiff_kappa", 1, 4, m.xyz, m.conn, dofs, rp, ci, kappa)
    kd = torch.from_numpy(kappa).cuda()
    v64 = b.assemble("stiff_kappa", coeff=kd, quad=4, prec="f64")
    b.status()
    assert row_scaled_err(rp, ref, v64.cpu().numpy()) <= F64_TOL
    v32 = b.assemble("stiff_kappa", coeff=kd, quad=4, prec="f32")
    assert row_scaled_err(rp, ref, v32.cpu().numpy()) <= F32_TOL
    x = np.random.default_rng(1).uniform(-1, 1, b.ndof)
    y_ref = orc.spmv(rp, ci, ref, x)
    xd = torch.from_numpy(x).cuda()
    y = b.apply(v64, xd)
    ys = [b.apply(v64, xd) for _ in range(100)]
    assert all(torch.equal(y, yk) for yk in ys)
    yh = y.cpu().numpy()
    row_abs = orc.spmv(rp, ci, np.abs(ref), np.abs(x))  # sum_j |A_ij x_j|: the scale of each row's sum
    # the SpMV arithmetic alone (the oracle's SpMV of the GPU's values) ...
    y_same = orc.spmv(rp, ci, v64.cpu().numpy(), x)
    assert np.max(np.abs(yh - y_same) / np.maximum(row_abs, 1e-300)) <= 1e-13
    # ... and against the oracle's operator (values within 1e-12 row-scaled)
    assert np.max(np.abs(yh - y_ref) / np.maximum(row_abs, 1e-300)) <= 1e-11


def test_p2_48cube_parity_and_solves():
    n = 48
    m = meshgen.kuhn_cube(n)
    kappa = meshgen.lognormal(len(m.conn), 0.5, 1)
    mesh = mg.Mesh(m.xyz, m.conn, order=2)
    b = mg.MatrixBuilder(mesh)
    assert (b.ndof, b.nnz) == (912673, 25755265)
    en, ee = orc.edges(len(m.xyz), m.conn, "lex")
    dofs = orc.elem_dofs(2, len(m.xyz), m.conn, ee)
    assert np.array_equal(mesh.elem_dofs(), dofs)
    rp, ci = orc.pattern(2, b.ndof, dofs)
    rph, cih = b.pattern()
    assert np.array_equal(rph, rp) and np.array_equal(cih, ci)
    ref = orc.assemble("stiff_kappa", 2, 15, m.xyz, m.conn, dofs, rp, ci, kappa)
    kd = torch.from_numpy(kappa).cuda()
    A64 = b.assemble("stiff_kappa", coeff=kd, quad=11, prec="f64")
    b.status()
    assert row_scaled_err(rp, ref, A64.cpu().numpy()) <= F64_TOL
    A32 = b.assemble("stiff_kappa", coeff=kd, quad=11, prec="f32")
    assert row_scaled_err(rp, ref, A32.cpu().numpy()) <= 2 * F32_TOL
    # the oracle's Dirichlet system and its exact discrete solution u_I
    X = np.concatenate([m.xyz, 0.5 * (m.xyz[en[:, 0]] + m.xyz[en[:, 1]])])
    bmask = meshgen.p2_boundary(m.boundary, en)
    uI = np.sin(np.pi * X[:, 0]) * np.sin(np.pi * X[:, 1]) * np.sin(np.pi * X[:, 2])
    uI[bmask] = 0.0
    K = ref.copy()
    orc.apply_dirichlet(rp, ci, bmask, K)
    rhs = orc.spmv(rp, ci, K, uI)
    mask = torch.from_numpy(bmask)
    b.apply_dirichlet(A64, mask)
    b.apply_dirichlet(A32, mask)
    rd = torch.from_numpy(rhs).cuda()
    uId = torch.from_numpy(uI).cuda()
    x64, i64 = b.cg(A64, rd, rtol=1e-10, maxit=50000)
    xmx, imx = b.cg_refined(A64, A32, rd, rtol=1e-10, inner_rtol=1e-2)
    assert i64.converged and imx.converged
    err64 = float(torch.linalg.norm(x64 - uId) / torch.linalg.norm(uId))
    errmx = float(torch.linalg.norm(xmx - uId) / torch.linalg.norm(uId))
    print(f"P2 48^3 error vs the oracle system's exact solution: FP64 CG {err64:.2e} ({i64.iterations} it), "
          f"mixed {errmx:.2e} ({imx.iterations} it, {imx.outer_iterations} anchors)")
    assert err64 <= 1e-8 and errmx <= 1e-8


def test_p1_128cube_pattern_and_sampled_rows():
    m = meshgen.kuhn_cube(128, jitter=0.25, seed=3, permute=True)
    kappa = meshgen.lognormal(len(m.conn), 1.5, 3)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    assert (b.ndof, b.nnz) == (2146689, 31802497)
    dofs = orc.elem_dofs(1, len(m.xyz), m.conn)
    rp, ci = orc.pattern(1, len(m.xyz), dofs)
    rph, cih = b.pattern()
    assert np.array_equal(rph, rp) and np.array_equal(cih, ci)
    del cih
    rows = np.sort(np.random.default_rng(7).choice(b.ndof, 16384, replace=False))
    touched = np.zeros(b.ndof, dtype=bool)
    touched[rows] = True
    sel = np.nonzero(touched[m.conn].any(axis=1))[0]  # every element touching a sampled row, element order
    conn_s = np.ascontiguousarray(m.conn[sel])
    ref = orc.assemble("stiff_kappa", 1, 4, m.xyz, conn_s, np.ascontiguousarray(dofs[sel]), rp, ci,
                       np.ascontiguousarray(kappa[sel]))
    kd = torch.from_numpy(kappa).cuda()
    v64 = b.assemble("stiff_kappa", coeff=kd, quad=4, prec="f64")
    b.status()
    assert _rows_err(rp, rows, ref, v64.cpu().numpy()) <= F64_TOL
    del v64
    v32 = b.assemble("stiff_kappa", coeff=kd, quad=4, prec="f32")
    assert _rows_err(rp, rows, ref, v32.cpu().numpy()) <= F32_TOL
