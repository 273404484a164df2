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


def expected_slot_map(order, elem_order, dofs, rowptr, colind):
    """The slot map of the gather assembly restated: for every diagonal or upper CSR
    entry (r, c) in CSR order, its mirror (c, r) and the element-matrix entries of
    every element holding both dofs, in ascending Morton position p, each
    p * nu + u (P1, element-major) or u * E + p (P2), u = sym_index of the pair."""
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
    useg, uslot, umirror, src = [0], [], [], []
    for r in range(len(rowptr) - 1):
        for k in range(rowptr[r], rowptr[r + 1]):
            c = int(colind[k])
            if c < r:
                continue
            uslot.append(k)
            m0 = rowptr[c]
            umirror.append(m0 + int(np.searchsorted(colind[m0:rowptr[c + 1]], r)))
            src.extend(contrib.get((r, c), []))
            useg.append(len(src))
    return {"useg": np.array(useg, dtype=np.int32), "uslot": np.array(uslot, dtype=np.int32),
            "umirror": np.array(umirror, dtype=np.int32), "src": np.array(src, dtype=np.uint32)}


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
    flat = em.reshape(-1) if order == 1 else em.T.reshape(-1)
    out = np.full(nnz, np.nan)
    for t in range(len(sm["uslot"])):
        v = 0.0
        for s in sm["src"][sm["useg"][t]:sm["useg"][t + 1]]:
            v += flat[s]
        out[sm["uslot"][t]] = v
        out[sm["umirror"][t]] = v
    return out
