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


def emulate_schedule(sched, order, local_mats, nnz, rowptr):
    """Runs the assembly kernel's two phases on the host with given element
    matrices (local_mats[e] = [field i, test j]) -- checks the schedule only."""
    info = sched["info"]
    nb = 4 if order == 1 else 10
    nb2 = nb * nb
    CI, T, W = info.chunk_items, info.threads, info.warps
    out = np.zeros(nnz)
    blocks, items, cptr, ent = sched["blocks"], sched["items"], sched["chunk_ptr"], sched["entries"]
    rows, racc = sched["rows"], sched["row_acc"]
    for b in range(info.nblocks):
        ib, ic, cb, nc, rb, rc = (int(v) for v in blocks[b, :6])
        acc = np.zeros(info.acc_max)
        for c in range(nc):
            buf = np.zeros(CI * nb2 + 1)
            for t in range(min(CI, ic - c * CI)):
                e = items[ib + c * CI + t]
                buf[np.arange(nb2) * CI + t] = local_mats[e].reshape(-1)
            base = (cb + c) * (W + 1)
            for w in range(W):
                seg = ent[cptr[base + w]:cptr[base + w + 1]].reshape(-1, 32)
                for k in range(seg.shape[0]):
                    words = seg[k]
                    slot = (words >> 16).astype(np.int64) * T + 32 * w + np.arange(32)
                    acc[slot] += buf[(words & 0xffff).astype(np.int64)]
        for r in range(rc):
            row, a0 = rows[rb + r], racc[rb + r]
            ln = rowptr[row + 1] - rowptr[row]
            out[rowptr[row]:rowptr[row + 1]] = acc[a0:a0 + ln]
    return out
