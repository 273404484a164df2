"""The Epetra and Tpetra drop-in adapters (include/morgana_gpu_epetra.hpp,
include/morgana_gpu_tpetra.hpp) compiled against test doubles of the Trilinos
classes they touch (tests/adapter/mock_trilinos): on CPU that they compile and
that the builders hand every row of K and B over; on
the GPU that the operator they hand to the Trilinos side (rows inserted into the
Epetra_FECrsMatrix, the same rows into the Tpetra::CrsMatrix, Apply through the
Epetra_Operator seam) is the oracle's."""
import os
import subprocess

import numpy as np
import pytest

from morganapublic_gb300 import build as mgbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "adapter", "adapter_check.cpp")
FLAGS = ["-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
         "-I" + os.path.join(ROOT, "tests", "adapter", "mock_trilinos"),
         "-I" + os.path.join(mgbuild.CUDA_HOME, "include")]


def test_adapter_compiles(tmp_path):
    subprocess.run(["g++", *FLAGS, "-Wall", "-Werror", "-c", SRC, "-o", str(tmp_path / "a.o")], check=True)


@pytest.mark.parametrize("test_order", [0, 1, 2])
@pytest.mark.parametrize("order", [1, 2])
def test_rows_reach_epetra_and_tpetra(tmp_path, order, test_order):
    """buildEpetraCrs / buildTpetraCrs (K) and buildEpetraLagrange /
    buildTpetraLagrange (B) on the host: every row, with the maps the
    reference's builder gives B (domain = field, range = multipliers).  Values
    come from host definitions of mg_assemble_host and mg_lagrange_assemble_host
    in the check itself, so no device is needed."""
    from morganapublic_gb300 import meshgen
    lib = mgbuild.build()
    src = os.path.join(ROOT, "tests", "adapter", "rows_check.cpp")
    exe = str(tmp_path / "rows_check")
    subprocess.run(["g++", *FLAGS, "-Wall", "-Werror", src, "-o", exe, lib,
                    "-L" + os.path.join(mgbuild.CUDA_HOME, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.dirname(lib),
                    "-Wl,-rpath," + os.path.join(mgbuild.CUDA_HOME, "lib64")], check=True)
    m = meshgen.kuhn_cube(3, jitter=0.2, seed=33, permute=True)
    with open(tmp_path / "in.bin", "wb") as f:
        np.array([len(m.xyz), len(m.conn), order], dtype=np.int64).tofile(f)
        m.xyz.astype(np.float64).tofile(f)
        m.conn.astype(np.int32).tofile(f)
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(test_order)], timeout=120)
    assert r.returncode == 0, r.returncode


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_adapter_against_oracle(tmp_path, order):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oracle as orc
    from morganapublic_gb300 import meshgen
    from helpers import row_scaled_err
    lib = mgbuild.build()
    exe = str(tmp_path / "adapter_check")
    subprocess.run(["g++", *FLAGS, SRC, "-o", exe, lib, "-L" + os.path.join(mgbuild.CUDA_HOME, "lib64"),
                    "-lcudart", "-Wl,-rpath," + os.path.dirname(lib),
                    "-Wl,-rpath," + os.path.join(mgbuild.CUDA_HOME, "lib64")], check=True)
    m = meshgen.kuhn_cube(4 if order == 1 else 3, jitter=0.2, seed=31, permute=True)
    kappa = meshgen.lognormal(len(m.conn), 1.0, 31)
    dofs, rp, ci, ref = orc.full_operator("stiff_kappa", order, 4, m.xyz, m.conn, coeff=kappa)
    ndof = len(rp) - 1
    x = np.random.default_rng(2).uniform(-1, 1, ndof)
    with open(tmp_path / "in.bin", "wb") as f:
        np.array([len(m.xyz), len(m.conn), order], dtype=np.int64).tofile(f)
        m.xyz.astype(np.float64).tofile(f)
        m.conn.astype(np.int32).tofile(f)
        kappa.astype(np.float64).tofile(f)
        x.tofile(f)
    subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True, timeout=300)
    raw = open(tmp_path / "out.bin", "rb").read()
    nd, nz = np.frombuffer(raw[:16], dtype=np.int64)
    off = 16
    rp_g = np.frombuffer(raw[off:off + 4 * (nd + 1)], dtype=np.int32); off += 4 * (nd + 1)
    ci_g = np.frombuffer(raw[off:off + 4 * nz], dtype=np.int32); off += 4 * nz
    va_g = np.frombuffer(raw[off:off + 8 * nz], dtype=np.float64); off += 8 * nz
    y_g = np.frombuffer(raw[off:off + 8 * nd], dtype=np.float64)
    assert nd == ndof and np.array_equal(rp_g, rp) and np.array_equal(ci_g, ci)
    assert row_scaled_err(rp, ref, va_g) <= 1e-12
    y_ref = orc.spmv(rp, ci, ref, x)
    assert np.max(np.abs(y_g - y_ref)) <= 1e-12 * np.abs(y_ref).max()
