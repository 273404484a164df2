"""Shared helpers of the parity tests (test-side only)."""
import numpy as np


def row_scaled_err(rowptr, ref_vals, vals):
    """max over entries of |a - b| / max(|a|, max_j |A_row,j|): the row-scaled error
    used for FP64 value parity (exact cancellations make some entries ~0)."""
    ref_vals = np.asarray(ref_vals, dtype=np.float64)
    vals = np.asarray(vals, dtype=np.float64)
    nrows = len(rowptr) - 1
    lens = np.diff(rowptr)
    row_of = np.repeat(np.arange(nrows), lens)
    rowmax = np.zeros(nrows)
    np.maximum.at(rowmax, row_of, np.abs(ref_vals))
    scale = np.maximum(np.abs(ref_vals), rowmax[row_of])
    scale[scale == 0] = 1.0
    return float(np.max(np.abs(ref_vals - vals) / scale)) if len(vals) else 0.0


def sym_index(i, j, nb):
    if i > j:
        i, j = j, i
    return i * nb - i * (i - 1) // 2 + (j - i)


def morton_elem_order(xyz, conn):
    """The assembly's element order restated: Morton keys (21 bits per axis over the
    nodes' bounding box) of the centroids 0.25 x_v summed over v in order, sorted by
    key, ties by element id."""
    xyz = np.asarray(xyz, dtype=np.float64)
    conn = np.asarray(conn, dtype=np.int64)
    if len(conn) == 0:
        return np.zeros(0, dtype=np.int32)
    lo, hi = xyz.min(axis=0), xyz.max(axis=0)
    c = np.zeros((len(conn), 3))
    for v in range(4):
        c = c + 0.25 * xyz[conn[:, v]]
    key = np.zeros(len(conn), dtype=np.uint64)
    for k in range(3):
        t = (c[:, k] - lo[k]) / (hi[k] - lo[k]) if hi[k] > lo[k] else np.zeros(len(conn))
        q = np.minimum(2097151.0, np.maximum(0.0, t * 2097151.0)).astype(np.uint64)
        spread = np.zeros(len(conn), dtype=np.uint64)
        for bit in range(21):
            spread |= ((q >> np.uint64(bit)) & np.uint64(1)) << np.uint64(3 * bit)
        key |= spread << np.uint64(k)
    return np.lexsort((np.arange(len(conn)), key)).astype(np.int32)


PAD_SOURCE = 0xFFFFFFFF


def expected_slot_map(order, elem_order, dofs, rowptr, colind, rows_per_block=256):
    """The slot map of the gather assembly restated.  For every diagonal or upper
    CSR entry (r, c): its mirror (c, r) and the element-matrix entries of every
    element holding both dofs, in ascending Morton position p, each p * nu + u
    (P1, element-major) or u * E + p (P2), u = sym_index of the pair.  Entries in
    groups of 32, ordered by (row // rows_per_block, off-diagonal, CSR position);
    a group's sources [j][lane], padded to its longest list with PAD_SOURCE."""
    nb = 4 if order == 1 else 10
    nu = nb * (nb + 1) // 2
    E = len(elem_order)
    dm = np.asarray(dofs)[np.asarray(elem_order)]
    contrib = {}
    for p in range(E):
        for i in range(nb):
            for j in range(nb):
                r, c = int(dm[p, i]), int(dm[p, j])
                if c >= r:
                    u = sym_index(i, j, nb)
                    contrib.setdefault((r, c), []).append(p * nu + u if order == 1 else u * E + p)
    keyed = []
    for r in range(len(rowptr) - 1):
        for k in range(rowptr[r], rowptr[r + 1]):
            c = int(colind[k])
            if c < r:
                continue
            m0 = rowptr[c]
            entry = (k, m0 + int(np.searchsorted(colind[m0:rowptr[c + 1]], r)), contrib.get((r, c), []))
            keyed.append(((r // rows_per_block, c != r, k), entry))
    keyed.sort(key=lambda x: x[0])
    entries = [e for _, e in keyed]
    n_diag = sum(1 for key, _ in keyed if not key[1])
    goff, src = [0], []
    for g in range(0, len(entries), 32):
        grp = entries[g:g + 32]
        L = max(len(e[2]) for e in grp)
        block = np.full((L, 32), PAD_SOURCE, dtype=np.uint64)
        for lane, e in enumerate(grp):
            block[:len(e[2]), lane] = e[2]
        src.extend(block.reshape(-1).tolist())
        goff.append(len(src))
    return {"goff": np.array(goff, dtype=np.int32), "uslot": np.array([e[0] for e in entries], dtype=np.int32),
            "umirror": np.array([e[1] for e in entries], dtype=np.int32), "src": np.array(src, dtype=np.uint32),
            "n_diag": n_diag}


def emulate_slot_map(sm, order, elem_order, local_mats, nnz):
    """The gather assembly run on the host with given element matrices
    (local_mats[e] = [field i, test j]) through a slot map -- checks the map only."""
    nb = 4 if order == 1 else 10
    nu = nb * (nb + 1) // 2
    E = len(elem_order)
    em = np.zeros((E, nu))
    pairs = [(i, j) for i in range(nb) for j in range(i, nb)]
    for p, e in enumerate(elem_order):
        for u, (i, j) in enumerate(pairs):
            em[p, u] = local_mats[e][i, j]
    flat = np.append(em.reshape(-1) if order == 1 else em.T.reshape(-1), 0.0)
    out = np.full(nnz, np.nan)
    U = len(sm["uslot"])
    for g in range(len(sm["goff"]) - 1):
        blk = sm["src"][sm["goff"][g]:sm["goff"][g + 1]].reshape(-1, 32)
        for lane in range(32):
            t = 32 * g + lane
            if t >= U:
                continue
            v = 0.0
            for s in blk[:, lane]:
                v += flat[min(int(s), len(flat) - 1)]
            out[sm["uslot"][t]] = v
            out[sm["umirror"][t]] = v
    return out


NO_OUTPUT = -2**31


def expected_block_map(elem_order, dofs, rowptr, colind, elems_per_block=512):
    """The block map of the one-pass P1 assembly restated.  Upper entries (r, c),
    c >= r, in CSR order; an entry's sources are p * 10 + u for every element p
    (Morton position) holding both dofs, ascending p.  A run is a maximal stretch
    of them in one block (p // elems_per_block); an entry with one run is complete,
    else shared (an entry without sources is one empty run of block 0).  Runs
    sorted stably by (block, longest first, lengths from 63 up tied) and cut
    into groups of 32 per block; a group's local sources (p - b Be) * 10 + u stored [j][lane], padded
    with Be * 10; outputs (slot, mirror) for a complete entry, (-1 - q, 0) for
    partial slot q, (NO_OUTPUT, 0) for an empty lane.  Shared entries sorted
    stably by run count (most first, 63 and more tied), groups of 32, run j of
    lane l at slot sgoff[g] + 32 j + l."""
    nb, nu, Be = 4, 10, elems_per_block
    E = len(elem_order)
    nblk = max(1, (E + Be - 1) // Be)
    dm = np.asarray(dofs)[np.asarray(elem_order)]
    contrib = {}
    for p in range(E):
        for i in range(nb):
            for j in range(nb):
                r, c = int(dm[p, i]), int(dm[p, j])
                if c >= r:
                    contrib.setdefault((r, c), []).append(p * nu + sym_index(i, j, nb))
    entries = []  # (slot, mirror, sources)
    for r in range(len(rowptr) - 1):
        for k in range(rowptr[r], rowptr[r + 1]):
            c = int(colind[k])
            if c < r:
                continue
            m0 = rowptr[c]
            mirror = m0 + int(np.searchsorted(colind[m0:rowptr[c + 1]], r))
            entries.append((k, mirror, contrib.get((r, c), [])))
    runs_of = []
    for slot, mirror, srcs in entries:
        runs = []
        for s in srcs:
            b = (s // nu) // Be
            if runs and runs[-1][0] == b:
                runs[-1][1].append(s)
            else:
                runs.append((b, [s]))
        runs_of.append(runs if runs else [(0, [])])
    shared = [t for t in range(len(entries)) if len(runs_of[t]) > 1]
    shared.sort(key=lambda t: 63 - min(len(runs_of[t]), 63))  # stable: most runs first, then CSR order
    sidx = {t: i for i, t in enumerate(shared)}
    sgoff, sout = [0], []
    for g in range(0, len(shared), 32):
        grp = shared[g:g + 32]
        sgoff.append(sgoff[-1] + 32 * max(len(runs_of[t]) for t in grp))
        sout.extend([entries[t][0], entries[t][1]] for t in grp)
        sout.extend([NO_OUTPUT, NO_OUTPUT] for _ in range(32 - len(grp)))
    recs = []  # ((block, 63 - min(length, 63)), t, j, sources)
    for t, runs in enumerate(runs_of):
        for j, (b, srcs) in enumerate(runs):
            recs.append(((b, 63 - min(len(srcs), 63)), t, j, srcs))
    recs.sort(key=lambda x: x[0])  # stable: CSR order, then j, within a (block, length)
    by_block = [[] for _ in range(nblk)]
    for x in recs:
        by_block[x[0][0]].append(x)
    bgrp, goff, src, out = [], [0], [], []
    for b in range(nblk):
        bgrp.append(len(goff) - 1)
        if True:
            seg = by_block[b]
            for g in range(0, len(seg), 32):
                grp = seg[g:g + 32]
                L = max(len(x[3]) for x in grp)
                rows = np.full((L, 32), Be * nu, dtype=np.uint16)
                for lane, (_, t, j, srcs) in enumerate(grp):
                    rows[:len(srcs), lane] = [s - b * Be * nu for s in srcs]
                    if len(runs_of[t]) == 1:
                        out.append([entries[t][0], entries[t][1]])
                    else:
                        s_i = sidx[t]
                        out.append([-1 - (sgoff[s_i // 32] + 32 * j + s_i % 32), 0])
                out.extend([NO_OUTPUT, 0] for _ in range(32 - len(grp)))
                src.extend(rows.reshape(-1).tolist())
                goff.append(len(src))
    bgrp.append(len(goff) - 1)
    return {"bgrp": np.array(bgrp, dtype=np.int32), "goff": np.array(goff, dtype=np.int32),
            "src": np.array(src, dtype=np.uint16), "out": np.array(out, dtype=np.int32).reshape(-1, 2),
            "sgoff": np.array(sgoff, dtype=np.int32), "sout": np.array(sout, dtype=np.int32).reshape(-1, 2),
            "n_shared": len(shared), "n_runs": len(recs), "n_upper": len(entries)}


def emulate_block_map(bm, elem_order, local_mats, nnz, elems_per_block=None):
    """The one-pass P1 assembly run on the host with given element matrices
    (local_mats[e] = [field i, test j]) through a block map -- checks the map only:
    per block its local sums (complete entries written, shared ones to their
    partial slots), then the partial sums in slot order."""
    nu = 10
    Be = int(bm["info"].elems_per_block if elems_per_block is None else elems_per_block)
    pairs = [(i, j) for i in range(4) for j in range(i, 4)]
    E = len(elem_order)
    em = np.zeros((max(1, (E + Be - 1) // Be) * Be, nu))
    for p, e in enumerate(elem_order):
        for u, (i, j) in enumerate(pairs):
            em[p, u] = local_mats[e][i, j]
    values = np.full(nnz, np.nan)
    partial = np.zeros(max(1, int(bm["sgoff"][-1])))
    for b in range(len(bm["bgrp"]) - 1):
        local = np.append(em[b * Be:(b + 1) * Be].reshape(-1), 0.0)
        for g in range(bm["bgrp"][b], bm["bgrp"][b + 1]):
            rows = bm["src"][bm["goff"][g]:bm["goff"][g + 1]].reshape(-1, 32)
            for lane in range(32):
                v = 0.0
                for s in rows[:, lane]:
                    v += local[int(s)]
                o = bm["out"][32 * g + lane]
                if o[0] >= 0:
                    values[o[0]] = v
                    values[o[1]] = v
                elif o[0] != NO_OUTPUT:
                    partial[-1 - o[0]] = v
    for g in range(len(bm["sgoff"]) - 1):
        rows = partial[bm["sgoff"][g]:bm["sgoff"][g + 1]].reshape(-1, 32)
        for lane in range(32):
            o = bm["sout"][32 * g + lane]
            if o[0] >= 0:
                v = 0.0
                for x in rows[:, lane]:
                    v += x
                values[o[0]] = values[o[1]] = v
    return values


def _oriented(xyz, conn):
    """conn with each tet's last two vertices swapped where its determinant is negative."""
    conn = np.array(conn, dtype=np.int32)
    e = xyz[conn[:, 1:]] - xyz[conn[:, :1]]
    neg = np.linalg.det(e) < 0
    conn[neg, 2], conn[neg, 3] = conn[neg, 3].copy(), conn[neg, 2].copy()
    return conn


def star_mesh(n_points=700, seed=0):
    """Tetrahedra joining a centre node to the hull triangles of points on a sphere
    (all of them on the hull: 2 n_points - 4 elements): every element holds node 0
    (one node of very high valence)."""
    from scipy.spatial import ConvexHull
    k = np.arange(n_points) + 0.5
    phi = np.arccos(1 - 2 * k / n_points)
    th = np.pi * (1 + 5 ** 0.5) * k
    pts = np.stack([np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)], axis=1)
    pts = pts @ np.linalg.qr(np.random.default_rng(seed).normal(size=(3, 3)))[0]  # a seeded rotation
    xyz = np.vstack([np.zeros((1, 3)), pts])
    tris = ConvexHull(pts).simplices + 1
    conn = np.hstack([np.zeros((len(tris), 1), dtype=np.int64), tris])
    return xyz, _oriented(xyz, conn)


def disjoint_tets(n_tets=1500, seed=0):
    """Tetrahedra sharing no node: every CSR entry has one source."""
    rng = np.random.default_rng(seed)
    base = rng.uniform(0, 10, (n_tets, 1, 3))
    ref = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    xyz = (base + ref[None] + 0.1 * rng.uniform(-1, 1, (n_tets, 4, 3))).reshape(-1, 3)
    conn = np.arange(4 * n_tets).reshape(n_tets, 4)
    return xyz, _oriented(xyz, conn)
