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
