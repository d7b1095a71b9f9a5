"""Multi-level meshblock ghost fill -- TEST INFRASTRUCTURE ONLY (the CPU
oracle; see oracle/__init__.py for who may use it).

Restates how load_athenak_meshblocks fills the one-cell ghost layer of each
meshblock on a mesh with refinement levels (mahakala/grmhd/athenak.py:
103-158 with _get_key_for_level :160-190, _get_slice_source /
_get_01_source :192-206 and _get_new_meshblock_boundary :208-525).  For a
ghost region (di, dj, dk) of a block at level L and logical location t, the
first of these that exists supplies it:

* the same-level neighbour t + d: a copy of its adjacent cells
  (athenak.py:211-229);
* the coarser neighbour at level L-1, location floor((t + d)/2): each of its
  cells copied into the 2 fine ghost cells it covers per transverse axis,
  the half of the coarse block chosen by the parity of t + d
  (athenak.py:232-289);
* the finer neighbours at level L+1 (2 (t + d), shifted by one for d = -1):
  the mean of 2x2x2 fine cells, accumulated term by term in float64 as
  value/8 of the float32 data (athenak.py:300-522).  In the edge case (two
  non-zero d) the reference's loop reads the transverse source as a
  single cell (index 0) for its first term and then as the every-other-cell
  slice selected by the PREVIOUS term's offset (athenak.py:439-459 assign
  the new slice to source_*, not copy_source_*); that order is kept here,
  since it decides the values;
* nothing: the ghosts stay zero (the domain edge).

Cubic blocks only (n cells per axis, n even), as the reference assumes.
"""

import itertools

import numpy as np


def _order():
    # the reference's term order: v1 (i) outermost, v3 (k) innermost
    return [(v1, v2, v3) for v1 in (0, 1) for v2 in (0, 1) for v3 in (0, 1)]


def multilevel_meshblocks(data, locs, levels):
    """data (8, nmb, n, n, n) float32 indexed [prim, mb, k, j, i]; locs
    (nmb, 3) = (i, j, k); levels (nmb,).  Returns the ghost-filled blocks
    (nmb, 8, n+2, n+2, n+2) float64 indexed [mb, prim, k, j, i]."""
    data = np.asarray(data, dtype=np.float32)
    _, nmb, n, _, _ = data.shape
    if n % 2:
        raise ValueError("the refinement rules need an even number of cells per block")
    h = n // 2
    key = {(int(levels[m]), int(locs[m][0]), int(locs[m][1]), int(locs[m][2])): m for m in range(nmb)}
    out = np.zeros((nmb, 8, n + 2, n + 2, n + 2))
    out[:, :, 1:-1, 1:-1, 1:-1] = data.transpose(1, 0, 2, 3, 4)
    eighth = np.float32(8.0)
    for m in range(nmb):
        lv = int(levels[m])
        t = [int(v) for v in locs[m]]
        for d in itertools.product((-1, 0, 1), repeat=3):
            if d == (0, 0, 0):
                continue
            # ghost coordinates (padded) per axis a = 0 (i), 1 (j), 2 (k)
            tgt = [np.array([n + 1]) if d[a] == 1 else (np.array([0]) if d[a] == -1 else np.arange(1, n + 1))
                   for a in range(3)]
            val = _region(data, key, lv, t, d, tgt, n, h, eighth)
            if val is not None:
                out[m][np.ix_(np.arange(8), tgt[2], tgt[1], tgt[0])] = val
    return out


def _gather(data, nb, src):
    """data[:, nb] at per-axis index arrays src = (i, j, k) -> (8, k, j, i)."""
    return data[:, nb][np.ix_(np.arange(8), src[2], src[1], src[0])]


def _region(data, key, lv, t, d, tgt, n, h, eighth):
    nb = key.get((lv, t[0] + d[0], t[1] + d[1], t[2] + d[2]))
    if nb is not None:  # same level
        src = [np.array([0]) if d[a] == 1 else (np.array([n - 1]) if d[a] == -1 else tgt[a] - 1) for a in range(3)]
        return _gather(data, nb, src).astype(np.float64)
    nb = key.get((lv - 1, (t[0] + d[0]) // 2, (t[1] + d[1]) // 2, (t[2] + d[2]) // 2))
    if nb is not None:  # coarser neighbour: copy
        src = []
        for a in range(3):
            odd = (t[a] + d[a]) % 2
            if d[a] == 1:
                src.append(np.array([h if odd else 0]))
            elif d[a] == -1:
                src.append(np.array([n - 1 if odd else h - 1]))
            else:
                src.append((h if odd else 0) + (tgt[a] - 1) // 2)
        return _gather(data, nb, src).astype(np.float64)
    if (lv + 1, 2 * (t[0] + d[0]), 2 * (t[1] + d[1]), 2 * (t[2] + d[2])) not in key:
        return None  # domain edge: zeros
    # finer neighbours: mean of 2x2x2 fine cells, one fine block per target cell
    base = [2 * (t[a] + d[a]) + (1 if d[a] == -1 else 0) for a in range(3)]
    s0 = [n - 2 if d[a] == -1 else 0 for a in range(3)]
    zero = [a for a in range(3) if d[a] == 0]
    edge = len(zero) == 1
    shape = (8, len(tgt[2]), len(tgt[1]), len(tgt[0]))
    val = np.zeros(shape)
    # per target cell along a zero axis: which fine block (ep) and which pair (mz)
    ep = {a: (tgt[a] - 1) // h for a in zero}
    mz = {a: (tgt[a] - 1) - ep[a] * h for a in zero}
    # the fine blocks: one per combination of edge positions
    eps = [sorted(set(ep[a].tolist())) if a in zero else [0] for a in range(3)]
    for e in itertools.product(*eps):
        nb = key[(lv + 1, base[0] + e[0], base[1] + e[1], base[2] + e[2])]
        sel = [np.nonzero(ep[a] == e[a])[0] if a in zero else np.arange(1) for a in range(3)]
        acc = np.zeros((8, len(sel[2]), len(sel[1]), len(sel[0])))
        prev = None
        for step, v in enumerate(_order()):
            src = []
            for a in range(3):
                if a not in zero:
                    src.append(np.array([s0[a] + v[a]]))
                elif edge and step == 0:
                    src.append(np.zeros(len(sel[a]), dtype=np.int64))   # one cell, broadcast
                elif edge:
                    src.append(prev[a] + 2 * mz[a][sel[a]])             # the previous term's offset
                else:
                    src.append(v[a] + 2 * mz[a][sel[a]])
            acc += (_gather(data, nb, src) / eighth).astype(np.float64)
            prev = v
        val[np.ix_(np.arange(8), sel[2], sel[1], sel[0])] = acc
    return val
