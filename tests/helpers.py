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


def decode_pieces(words, order):
    """The 8-byte contribution pieces of one warp's word range ([piece][lane], two
    32-bit words each, the lower first) as (slot, sources) arrays of shape
    (pieces, 32) and (pieces, 32, srcs): P1 four 12-bit sources at bits 0, 12,
    24, 36 and the slot at bit 48; P2 two words source (13 bits) | slot << 13."""
    w = np.asarray(words, dtype=np.uint64).reshape(-1, 32, 2)
    pc = w[:, :, 0] | (w[:, :, 1] << np.uint64(32))
    if order == 1:
        srcs = np.stack([(pc >> np.uint64(12 * k)) & np.uint64(0xfff) for k in range(4)], axis=-1)
        slot = (pc >> np.uint64(48)) & np.uint64(0x3fff)
    else:
        srcs = np.stack([w[:, :, 0] & np.uint64(0x1fff), w[:, :, 1] & np.uint64(0x1fff)], axis=-1)
        slot = (w[:, :, 0] >> np.uint64(13)) & np.uint64(0x3fff)
        assert np.array_equal(slot, (w[:, :, 1] >> np.uint64(13)) & np.uint64(0x3fff))
    return slot.astype(np.int64), srcs.astype(np.int64)


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
                # [piece][lane]: a piece's sources go to its slot
                slots, srcs = decode_pieces(ent[cptr[base + w]:cptr[base + w + 1]], order)
                for lane in range(32):
                    for slot, src in zip(slots[:, lane], srcs[:, lane]):
                        v = buf[src[0]]
                        for x in src[1:]:
                            v += buf[x]
                        acc[slot] += v
        for r in range(rc):
            row, a0 = rows[rb + r], racc[rb + r]
            ln = rowptr[row + 1] - rowptr[row]
            out[rowptr[row]:rowptr[row + 1]] = acc[a0:a0 + ln]
    return out
