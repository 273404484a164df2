"""Generates the golden fixtures in this directory from the reference's own
test data, read as text from a morganaPublic checkout (its path is the
required first argument).

  mignon3dC.json         tests/morganaMeshes/mignon3dC.msh: 7 nodes, 8 tets
                         (file order, node ids as written, geoId = 2nd tag)
                         and its boundary triangles with their geoIds
  mignon3dB.json         tests/morganaMeshes/mignon3dB.msh, the same way (the
                         mesh of localMatrixLA3dTest1, whose multipliers live
                         on the triangles of geoId 2)
  connect3d_edges.json   tests/morganaGeometry/logs/connect3dTest2.log: the
                         rank-0 element's local edges in lid order with their
                         node pair as stored (first-appearance enumeration)
  dofmap_counts.json     tests/morganaFields/logs/dofMapStatic3dTest{4,5,6,8}.log:
                         the largest global dof id printed for P1 / P0 / P2 on
                         mignon3dC, i.e. the global dof counts

Run: python tests/golden/make_golden.py <morganaPublic checkout>
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py <morganaPublic checkout>")
REF = sys.argv[1]
OUT = os.path.dirname(os.path.abspath(__file__))


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def mesh_fixture(name="mignon3dC"):
    lines = read(f"tests/morganaMeshes/{name}.msh").splitlines()
    i = next(k for k, l in enumerate(lines) if l.strip() == "$Nodes")
    n = int(lines[i + 1])
    nodes = [[float(v) for v in lines[i + 2 + k].split()[1:4]] for k in range(n)]
    j = next(k for k, l in enumerate(lines) if l.strip() == "$Elements")
    m = int(lines[j + 1])
    tets, geo, tris, tgeo = [], [], [], []
    for k in range(m):
        v = [int(t) for t in lines[j + 2 + k].split()]
        ntags = v[2]
        if v[1] == 4:
            tets.append(v[3 + ntags:3 + ntags + 4])
            geo.append(v[4])
        elif v[1] == 2:
            tris.append(v[3 + ntags:3 + ntags + 3])
            tgeo.append(v[4])
    return {"source": f"tests/morganaMeshes/{name}.msh", "nodes": nodes, "tets_1based": tets,
            "geo_ids": geo, "triangles_1based": tris, "triangle_geo_ids": tgeo}


def edge_fixture():
    text = read("tests/morganaGeometry/logs/connect3dTest2.log")
    sec = text.split("Edges---------------------------------------------------", 1)[1].split("COL", 1)[0]
    lids = [int(x) for x in re.findall(r"pid: 0 lid: (\d+)", sec)]
    conns = [[int(t) for t in c.split()] for c in re.findall(r"Connected Id's : ([\d ]+)", sec)]
    return {"source": "tests/morganaGeometry/logs/connect3dTest2.log (rank 0, one tet with local nodes 1 2 3 4)",
            "lids": lids, "edge_nodes_local_1based": conns}


def dof_counts():
    out = {"source": "tests/morganaFields/logs/dofMapStatic3dTest{4,5,6,8}.log (mignon3dC)"}
    for name, test in (("P1", 4), ("P0", 5), ("P2", 6), ("P2_b", 8)):
        text = read(f"tests/morganaFields/logs/dofMapStatic3dTest{test}.log")
        dm = text.split("Dof Map", 1)[1].split("List Map", 1)[0]
        out[name] = max(int(g) for g in re.findall(r"gid: (\d+)", dm))
    return out


if __name__ == "__main__":
    for name, data in (("mignon3dC.json", mesh_fixture("mignon3dC")), ("mignon3dB.json", mesh_fixture("mignon3dB")),
                       ("connect3d_edges.json", edge_fixture()), ("dofmap_counts.json", dof_counts())):
        with open(os.path.join(OUT, name), "w") as f:
            json.dump(data, f, indent=1)
        print("wrote", name)
