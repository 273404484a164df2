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


def emulate_schedule(sched, order, local_mats, nnz, rowptr):
    """Runs the assembly kernel's two phases on the host with given element
    matrices (local_mats[e] = [field i, test j]) -- checks the schedule only."""
    info = sched["info"]
    nb = 4 if order == 1 else 10
    nu = nb * (nb + 1) // 2
    pairs = [(i, j) for i in range(nb) for j in range(i, nb)]
    assert [sym_index(i, j, nb) for i, j in pairs] == list(range(nu))
    CI, W = info.chunk_items, info.warps
    out = np.zeros(nnz)
    blocks, items, cptr, ent = sched["blocks"], sched["items"], sched["chunk_ptr"], sched["entries"]
    rows, racc = sched["rows"], sched["row_acc"]
    for b in range(info.nblocks):
        ib, ic, cb, nc, rb, rc = (int(v) for v in blocks[b, :6])
        acc = np.zeros(info.acc_max + 1)  # + the padding words' dummy slot
        for c in range(nc):
            buf = np.zeros(nu * CI + 1)
            for t in range(min(CI, ic - c * CI)):
                e = items[ib + c * CI + t]
                for u, (i, j) in enumerate(pairs):
                    buf[u * CI + t] = local_mats[e][i, j]
            base = (cb + c) * (W + 1)
            for w in range(W):
                # [piece][lane][PW]: a piece's words go to the slot of its first word
                PW = 4 if order == 1 else 2
                seg = ent[cptr[base + w]:cptr[base + w + 1]].reshape(-1, 32, PW)
                for lane in range(32):
                    for piece in seg[:, lane, :]:
                        v = buf[int(piece[0]) & 0x1fff]
                        for word in piece[1:]:
                            v += buf[int(word) & 0x1fff]
                        acc[(int(piece[0]) >> 13) & 0x3fff] += v
        for r in range(rc):
            row, a0 = rows[rb + r], racc[rb + r]
            ln = rowptr[row + 1] - rowptr[row]
            out[rowptr[row]:rowptr[row + 1]] = acc[a0:a0 + ln]
    return out
