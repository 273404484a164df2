"""CPU tests of the product library's host side (no GPU calls): exported
symbols, mesh ingest, edge/dof numbering and CSR pattern against the oracle,
error paths, and the assembly's element order against its restatement."""
import json
import os
import re

import numpy as np
import pytest

import morganapublic_gb300 as mg
import oracle as orc
from morganapublic_gb300 import meshgen
from helpers import emulate_block_map, expected_block_map, morton_elem_order, row_scaled_err, star_mesh

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


@pytest.mark.parametrize("order,rule", [(1, "lex"), (2, "lex"), (2, "first")])
def test_high_valence_node_numbering_and_pattern(order, rule):
    """A node that starts 700 edges (every tet of a star mesh holds it): edge table,
    dof map and CSR pattern equal the oracle's -- no per-vertex or per-row limit."""
    xyz, conn = star_mesh(700, seed=3)
    mesh = mg.Mesh(xyz, conn, order=order, edge_rule=rule)
    ee = None
    ndof = len(xyz)
    if order == 2:
        en_o, ee = orc.edges(len(xyz), conn, rule)
        en, ee_p = mesh.edges()
        assert np.array_equal(en, en_o) and np.array_equal(ee_p, ee)
        ndof += len(en_o)
    dofs_o = orc.elem_dofs(order, len(xyz), conn, ee)
    assert mesh.ndof == ndof and np.array_equal(mesh.elem_dofs(), dofs_o)
    rp_o, ci_o = orc.pattern(order, ndof, dofs_o)
    rp, ci = mg.MatrixBuilder(mesh).pattern()
    assert np.array_equal(rp, rp_o) and np.array_equal(ci, ci_o)
    assert np.diff(rp).max() == ndof  # the centre couples with every dof


def test_pattern_sizes_of_survey_formulas():
    n = 4
    m = meshgen.kuhn_cube(n)
    b1 = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    nE = 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3
    assert b1.nnz == (n + 1) ** 3 + 2 * nE
    b2 = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=2))
    assert b2.nnz == 230 * n ** 3 + 138 * n ** 2 + 24 * n + 1


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("n,jitter,permute", [(3, 0.0, False), (5, 0.25, True)])
def test_elem_order_matches_restatement(order, n, jitter, permute):
    """The host plan's element order (a Morton curve of the centroids, ties by id)
    equals its numpy restatement, and is a permutation of the elements."""
    m = meshgen.kuhn_cube(n, jitter=jitter, seed=3, permute=permute)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=order))
    eo = b.elem_order()
    assert np.array_equal(np.sort(eo), np.arange(len(m.conn)))
    assert np.array_equal(eo, morton_elem_order(m.xyz, m.conn))


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


_PLAN_DUMP = r"""
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
    out[(n, order)] = (rp, ci, b.elem_order())
pickle.dump(out, open(sys.argv[2], "wb"))
"""


def test_plan_independent_of_thread_count(tmp_path):
    """The host plan (pattern and element order) is built with OpenMP; its
    per-thread counts and fills must give the same arrays for any thread count."""
    import pickle
    import subprocess
    import sys
    script = tmp_path / "dump.py"
    script.write_text(_PLAN_DUMP)
    res = {}
    for nth in (1, 4):
        env = dict(os.environ, OMP_NUM_THREADS=str(nth))
        out = tmp_path / f"s{nth}.pkl"
        subprocess.run([sys.executable, str(script), ROOT, str(out)], env=env, check=True, timeout=300)
        res[nth] = pickle.load(open(out, "rb"))
    for key, (rp, ci, eo) in res[1].items():
        rp4, ci4, eo4 = res[4][key]
        assert np.array_equal(rp, rp4) and np.array_equal(ci, ci4) and np.array_equal(eo, eo4)


@pytest.mark.parametrize("elems_per_block", [16, 64, 512])
def test_block_map_restatement_sums_to_oracle(elems_per_block):
    """The block-map restatement (the layout the GPU build is checked against) is
    self-consistent on CPU: with small blocks most entries span several blocks,
    and summing the oracle's element matrices through its local sums and partial
    slots gives the oracle's CSR values; every partial slot of a lane's runs is
    written exactly once, padding slots never."""
    m = meshgen.kuhn_cube(4, jitter=0.25, seed=4, permute=True)
    kappa = meshgen.lognormal(len(m.conn), 1.0, 9)
    b = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    rp, ci = b.pattern()
    order = b.elem_order()
    bm = expected_block_map(order, m.conn, rp, ci, elems_per_block)
    nblk = (len(m.conn) + elems_per_block - 1) // elems_per_block
    assert len(bm["bgrp"]) == nblk + 1 and (bm["n_shared"] > 0) == (nblk > 1)
    q = -1 - bm["out"][:, 0][(bm["out"][:, 0] < 0) & (bm["out"][:, 0] != -2**31)]
    assert len(q) == len(set(q.tolist())) == bm["n_runs"] - (bm["n_upper"] - bm["n_shared"])
    assert np.all(q < bm["sgoff"][-1])
    _, rpo, cio, ref = orc.full_operator("stiff_kappa", 1, 4, m.xyz, m.conn, coeff=kappa)
    mats = [orc.local_matrix("stiff_kappa", 1, 4, m.xyz, m.conn[e], kappa=kappa[e]) for e in range(len(m.conn))]
    got = emulate_block_map(bm, order, mats, b.nnz, elems_per_block)
    assert not np.isnan(got).any()
    assert row_scaled_err(rp, ref, got) <= 1e-14


def test_assembly_map_exports_refuse_the_other_order():
    """P1 plans assemble through the block map, P2 plans through the slot map: each
    export refuses the other kind with MG_ERR_UNSUPPORTED before any device work."""
    m = meshgen.kuhn_cube(2)
    b1 = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=1))
    b2 = mg.MatrixBuilder(mg.Mesh(m.xyz, m.conn, order=2))
    for call in (b1.slot_map_info, b1.export_slot_map, b2.block_map_info, b2.export_block_map):
        with pytest.raises(mg.MorganaError) as e:
            call()
        assert e.value.status == mg.MG_ERR_UNSUPPORTED
