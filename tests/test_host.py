"""CPU tests of the product library's host side (no GPU calls): exported
symbols, mesh ingest, edge/dof numbering and CSR pattern against the oracle,
error paths, and the assembly schedule emulated on the host."""
import json
import os
import re

import numpy as np
import pytest

import morganapublic_gb300 as mg
import oracle as orc
from morganapublic_gb300 import meshgen
from helpers import decode_pieces, emulate_schedule, row_scaled_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def header_functions():
    text = open(os.path.join(ROOT, "include", "morgana_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = mg.lib()
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
        assert n in mg.SIGNATURES, n
    assert mg.version().startswith("morgana-gb300")


@pytest.mark.parametrize("order,rule", [(1, "lex"), (2, "lex"), (2, "first")])
@pytest.mark.parametrize("n,jitter,permute", [(2, 0.0, False), (3, 0.2, True)])
def test_numbering_and_pattern_match_oracle(order, rule, n, jitter, permute):
    m = meshgen.kuhn_cube(n, jitter=jitter, seed=1, permute=permute)
    mesh = mg.Mesh(m.xyz, m.conn, order=order, edge_rule=rule)
    ee = None
    ndof = len(m.xyz)
    if order == 2:
        en_o, ee = orc.edges(len(m.xyz), m.conn, rule)
        en, ee_p = mesh.edges()
        assert np.array_equal(en, en_o)
        assert np.array_equal(ee_p, ee)
        ndof += len(en_o)
    dofs_o = orc.elem_dofs(order, len(m.xyz), m.conn, ee)
    assert mesh.ndof == ndof
    assert np.array_equal(mesh.elem_dofs(), dofs_o)
    builder = mg.MatrixBuilder(mesh)
    rp_o, ci_o = orc.pattern(order, ndof, dofs_o)
    rp, ci = builder.pattern()
    assert np.array_equal(rp, rp_o) and np.array_equal(ci, ci_o)
    assert abs(mesh.min_det - m.min_det) <= 1e-15 * abs(m.min_det) + 1e-300


def test_pattern_sizes_of_survey_formulas():
    n = 4
    m = meshgen.kuhn_cube(n)
    b1 = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    nE = 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3
    assert b1.nnz == (n + 1) ** 3 + 2 * nE
    b2 = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=2))
    assert b2.nnz == 230 * n ** 3 + 138 * n ** 2 + 24 * n + 1


@pytest.mark.parametrize("order,op,quad", [(1, "stiff_kappa", 4), (1, "mass", 4), (2, "stiff_kappa", 15),
                                           (2, "mass_coeff", 15)])
def test_schedule_emulation_matches_oracle(order, op, quad):
    """The exported schedule, run on the host with the oracle's element matrices,
    reproduces the oracle's CSR values (same terms; the per-slot association of
    the sum differs, so to a few ulps of the row)."""
    m = meshgen.kuhn_cube(3, jitter=0.2, seed=4, permute=True)
    kappa = meshgen.lognormal(len(m.conn), 1.0, 9)
    mesh = mg.Mesh(m.xyz, m.conn, order=order)
    builder = mg.MatrixBuilder(mesh)
    sched = builder.export_schedule()
    info = sched["info"]
    nb = 4 if order == 1 else 10
    assert info.n_contrib == len(m.conn) * nb * nb
    assert info.n_items >= len(m.conn)
    dofs, rp, ci, vals = orc.full_operator(op, order, quad, m.xyz, m.conn, coeff=kappa)
    mats = np.stack([orc.local_matrix(op, order, quad, m.xyz, m.conn[e], kappa=kappa[e]) for e in range(len(m.conn))])
    got = emulate_schedule(sched, order, mats, builder.nnz, rp)
    assert row_scaled_err(rp, vals, got) <= 1e-14


def test_schedule_covers_every_row_once():
    m = meshgen.kuhn_cube(4, permute=True, seed=3)
    builder = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=2))
    s = builder.export_schedule()
    assert np.array_equal(np.sort(s["rows"]), np.arange(builder.ndof))
    rp, _ = builder.pattern()
    for b in range(s["info"].nblocks):
        rb, rc, used = s["blocks"][b, 4], s["blocks"][b, 5], s["blocks"][b, 6]
        rows = s["rows"][rb:rb + rc]
        assert used == int(np.sum(rp[rows + 1] - rp[rows])) <= s["info"].acc_max


def test_gmsh_roundtrip(tmp_path):
    m = meshgen.kuhn_cube(3, jitter=0.25, seed=3, permute=True)
    p = str(tmp_path / "cube.msh")
    meshgen.write_gmsh(p, m.xyz, m.conn)
    mesh = mg.Mesh.load_gmsh(p, order=2)
    xyz, conn = mesh.geometry()
    assert np.array_equal(conn, m.conn)
    assert np.array_equal(xyz, m.xyz)  # %.17g round-trips doubles exactly


def test_gmsh_reference_mesh(tmp_path):
    """The reference's mignon3dC mesh (re-emitted from the golden fixture in the
    same Gmsh 2 layout): node ids by line order, tets in file order."""
    g = json.load(open(os.path.join(GOLDEN, "mignon3dC.json")))
    p = str(tmp_path / "mignon3dC.msh")
    nodes, tets, tris = g["nodes"], g["tets_1based"], g["triangles_1based"]
    with open(p, "w") as f:
        f.write("$MeshFormat\n2.1 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(nodes))
        for k, x in enumerate(nodes):
            f.write("%d %r %r %r\n" % (k + 1, *x))
        f.write("$EndNodes\n$Elements\n%d\n" % (len(tets) + len(tris)))
        k = 1
        for t in tris:
            f.write("%d 2 3 0 1 0 %d %d %d\n" % (k, *t))
            k += 1
        for t, gid in zip(tets, g["geo_ids"]):
            f.write("%d 4 3 0 %d 0 %d %d %d %d\n" % (k, gid, *t))
            k += 1
        f.write("$EndElements\n")
    mesh = mg.Mesh.load_gmsh(p, order=2, edge_rule="first")
    xyz, conn = mesh.geometry()
    assert np.array_equal(conn, np.array(tets) - 1)
    counts = json.load(open(os.path.join(GOLDEN, "dofmap_counts.json")))
    assert mesh.ndof == counts["P2"]


def test_bad_meshes_are_rejected():
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    with pytest.raises(mg.MorganaError) as e:
        mg.Mesh(xyz, np.array([[0, 2, 1, 3]], dtype=np.int32))  # inverted
    assert e.value.status == mg.MG_ERR_BAD_MESH
    with pytest.raises(mg.MorganaError) as e:
        mg.Mesh(xyz, np.array([[0, 1, 2, 7]], dtype=np.int32))  # node out of range
    assert e.value.status == mg.MG_ERR_BAD_MESH
    with pytest.raises(mg.MorganaError) as e:
        mg.Mesh(xyz, np.array([[0, 1, 1, 3]], dtype=np.int32))  # repeated node
    assert e.value.status == mg.MG_ERR_BAD_MESH
    with pytest.raises(mg.MorganaError) as e:
        mg.Mesh(xyz, np.array([[0, 1, 2, 3]], dtype=np.int32), order=3)
    assert e.value.status == mg.MG_ERR_INVALID_ARG
    with pytest.raises(mg.MorganaError) as e:
        mg.Mesh.load_gmsh("/nonexistent/file.msh")
    assert e.value.status == mg.MG_ERR_IO
    for bad in (np.nan, np.inf, -np.inf):  # non-finite coordinates, referenced or not
        for node in (3, 4):
            x = np.vstack([xyz, [[2.0, 2.0, 2.0]]])
            x[node, 2] = bad
            with pytest.raises(mg.MorganaError) as e:
                mg.Mesh(x, np.array([[0, 1, 2, 3]], dtype=np.int32))
            assert e.value.status == mg.MG_ERR_BAD_MESH


def test_empty_and_single_tet():
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    mesh = mg.Mesh(xyz, np.zeros((0, 4), dtype=np.int32))
    b = mg.MatrixBuilder(mesh)
    assert b.nnz == 0 and b.ndof == 4
    one = mg.MatrixBuilder(mg.Mesh(xyz, np.array([[0, 1, 2, 3]], dtype=np.int32), order=2))
    assert one.ndof == 10 and one.nnz == 100


def test_export_schedule_info_fields():
    m = meshgen.kuhn_cube(2)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn))
    info = b.schedule_info()
    assert info.threads == 256 and info.warps == 8 and info.acc_max == 8192 and info.host_copy == 1
    assert info.n_entries >= info.n_contrib
    s = b.export_schedule()
    # every block's item list is padded to a multiple of 4 with -1
    assert len(s["items"]) % 4 == 0 and (s["items"] >= -1).all()


@pytest.mark.parametrize("order", [1, 2])
def test_schedule_slots_have_one_writer_per_chunk(order):
    """Within a chunk each accumulator slot is written by exactly one thread (the
    kernel's race freedom); a piece's first word carries its slot and a real
    source; padding pieces target only the dummy slot with zero sources; real
    slots lie inside the block."""
    m = meshgen.kuhn_cube(4, jitter=0.2, seed=2, permute=True)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=order))
    s = b.export_schedule()
    info = s["info"]
    nu = 10 if order == 1 else 55
    zero = nu * info.chunk_items
    for bk in range(info.nblocks):
        cb, nc, used = s["blocks"][bk, 2], s["blocks"][bk, 3], s["blocks"][bk, 6]
        for c in range(cb, cb + nc):
            cp = s["chunk_ptr"][c * (info.warps + 1):(c + 1) * (info.warps + 1)]
            owner = {}
            PW = 4 if order == 1 else 2
            for w in range(info.warps):
                slots, srcl = decode_pieces(s["entries"][cp[w]:cp[w + 1]], order)
                assert srcl.shape[2] == PW
                for lane in range(32):
                    t = 32 * w + lane
                    for slot, srcs in zip(slots[:, lane], srcl[:, lane]):
                        slot, srcs = int(slot), [int(x) for x in srcs]
                        if slot == info.acc_max:
                            assert all(x == zero for x in srcs)
                            continue
                        assert slot < used and all(x <= zero for x in srcs) and srcs[0] < zero
                        assert owner.setdefault(slot, t) == t


_SCHEDULE_DUMP = r"""
import sys, pickle
import numpy as np
sys.path.insert(0, sys.argv[1])
import morganapublic_gb300 as mg
from morganapublic_gb300 import meshgen
out = {}
for n, order in ((12, 1), (5, 2)):
    m = meshgen.kuhn_cube(n, jitter=0.25, seed=3, permute=True)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=order))
    rp, ci = b.pattern()
    sched = b.export_schedule()
    out[(n, order)] = (rp, ci, {k: np.asarray(v) for k, v in sched.items() if k != "info"})
pickle.dump(out, open(sys.argv[2], "wb"))
"""


def test_plan_independent_of_thread_count(tmp_path):
    """The host plan (pattern and assembly schedule) is built with OpenMP; its
    per-thread counts and fills must give the same arrays for any thread count."""
    import pickle
    import subprocess
    import sys
    script = tmp_path / "dump.py"
    script.write_text(_SCHEDULE_DUMP)
    res = {}
    for nth in (1, 4):
        env = dict(os.environ, OMP_NUM_THREADS=str(nth))
        out = tmp_path / f"s{nth}.pkl"
        subprocess.run([sys.executable, str(script), ROOT, str(out)], env=env, check=True, timeout=300)
        res[nth] = pickle.load(open(out, "rb"))
    for key, (rp, ci, sched) in res[1].items():
        rp4, ci4, sched4 = res[4][key]
        assert np.array_equal(rp, rp4) and np.array_equal(ci, ci4)
        for name, arr in sched.items():
            assert np.array_equal(arr, sched4[name]), (key, name)
