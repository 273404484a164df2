"""The allocation-free CG entry point (mg_cg_solve_noalloc) against mg_cg_solve
and against the oracle's solution.

mg_cg_solve_noalloc is for callers that cannot allocate device memory during a
solve: host codes whose device memory belongs to another allocator (a caching
allocator or an arena sized at start-up) and time-stepping loops that must not
take the implicit synchronisation of cudaMalloc/cudaFree.  Its work space is a
fixed array inside the library, shared by every call.  This file is collected
last so that a `-x` run has already run every other test if it fails."""
import ctypes

import pytest

import morganapublic_gb300 as mg
import oracle as orc
from morganapublic_gb300 import meshgen

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def _system(n, seed):
    """P1 kappa-diffusion with f = 1 and Dirichlet u = 0 by symmetric elimination, on
    the GPU and (the same operator and right-hand side) in the oracle."""
    m = meshgen.kuhn_cube(n, jitter=0.2, seed=seed, permute=True)
    kappa = meshgen.lognormal(len(m.conn), 1.0, seed + 10)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    dofs = orc.elem_dofs(1, len(m.xyz), m.conn)
    rp, ci = orc.pattern(1, len(m.xyz), dofs)
    K = orc.assemble("stiff_kappa", 1, 4, m.xyz, m.conn, dofs, rp, ci, kappa)
    rhs = orc.assemble_rhs(1, 4, m.xyz, m.conn, dofs, b.ndof)
    v = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64")  # also makes the plan device-resident
    bt = torch.from_numpy(rhs).cuda()  # a copy: the oracle's elimination below works on the host arrays
    b.apply_dirichlet(v, torch.from_numpy(m.boundary), bt)
    orc.apply_dirichlet(rp, ci, m.boundary, K, rhs)
    x_orc, _, _, _ = orc.cg(rp, ci, K, rhs, rtol=1e-13)
    return b, v, bt, x_orc


def _noalloc(b, v, bt, rtol, maxit, x=None):
    x = torch.zeros_like(bt) if x is None else x
    info = mg.CgInfo()
    st = mg.lib().mg_cg_solve_noalloc(b._h, v.data_ptr(), bt.data_ptr(), x.data_ptr(), rtol, maxit,
                                      mg.PRECOND["jacobi"], ctypes.byref(info),
                                      torch.cuda.current_stream().cuda_stream)
    return st, x, info


def test_noalloc_cg_matches_cg_and_oracle_twice():
    b, v, bt, x_orc = _system(10, 3)
    x_ref, info_ref = b.cg(v, bt, rtol=1e-10, precond="jacobi")
    x_orc = torch.from_numpy(x_orc).cuda()
    for _ in range(2):  # the shared work array keeps the previous call's contents
        st, x, info = _noalloc(b, v, bt, 1e-10, 10000)
        assert st == mg.MG_OK, mg.lib().mg_last_error().decode()
        assert info.converged and info.rel_residual <= 1e-10
        assert info.iterations == info_ref.iterations
        assert float(torch.linalg.norm(x - x_ref) / torch.linalg.norm(x_ref)) <= 1e-12
        # the FP64 oracle's solution (its own CG to 1e-13) at the solve tolerance
        assert float(torch.linalg.norm(x - x_orc) / torch.linalg.norm(x_orc)) <= 1e-8
    # a different system through the same array right after
    b2, v2, bt2, x2_orc = _system(7, 5)
    x2_ref, _ = b2.cg(v2, bt2, rtol=1e-10)
    st, x2, _ = _noalloc(b2, v2, bt2, 1e-10, 10000)
    assert st == mg.MG_OK
    assert float(torch.linalg.norm(x2 - x2_ref) / torch.linalg.norm(x2_ref)) <= 1e-12
    x2_orc = torch.from_numpy(x2_orc).cuda()
    assert float(torch.linalg.norm(x2 - x2_orc) / torch.linalg.norm(x2_orc)) <= 1e-8


def test_noalloc_cg_leaves_device_memory_alone():
    """A warm call changes the device's free memory by nothing: no allocation in the solve."""
    b, v, bt, _ = _system(8, 4)
    st, _, _ = _noalloc(b, v, bt, 1e-10, 10000)  # first call on the device: symbol lookup
    assert st == mg.MG_OK
    x = torch.zeros_like(bt)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    st, x, info = _noalloc(b, v, bt, 1e-10, 10000, x=x)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert st == mg.MG_OK and info.converged
    assert free1 == free0


def test_noalloc_cg_zero_rhs():
    """b = 0: the solution is 0 and the reported residual is 0 (not NaN)."""
    b, v, bt, _ = _system(6, 2)
    zero = torch.zeros_like(bt)
    st, x, info = _noalloc(b, v, zero, 1e-10, 100)
    assert st == mg.MG_OK, mg.lib().mg_last_error().decode()
    assert info.converged and info.rel_residual == 0.0
    assert float(torch.abs(x).max()) == 0.0


def test_noalloc_cg_rejects_sizes_above_the_limit():
    n = 37  # P2 on 37^3 cells: (2n + 1)^3 = 421,875 dofs > MG_CG_NOALLOC_MAX_NDOF = 400,000
    m = meshgen.kuhn_cube(n)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=2))
    assert b.ndof > 400000
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    info = mg.CgInfo()
    st = mg.lib().mg_cg_solve_noalloc(b._h, dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), 1e-10, 10,
                                      1, ctypes.byref(info), None)
    assert st == mg.MG_ERR_SIZE
    assert "MG_CG_NOALLOC_MAX_NDOF" in mg.lib().mg_last_error().decode()
