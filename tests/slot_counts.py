"""Expected CSR slot multiplicities of the element scatter (shared by the CPU
and GPU tests of the colouring's race check)."""
import numpy as np


def explicit_counts(nelem, rowptr, cols, p=2):
    """Element loop: +1 for every (row, column) pair of every element."""
    nb = [n + p for n in nelem]
    ndof = 3 * nb[0] * nb[1] * nb[2]
    rowidx = np.repeat(np.arange(ndof), np.diff(rowptr))
    keys_csr = rowidx.astype(np.int64) * ndof + cols
    counts = np.zeros(len(cols))
    q = p + 1
    loc = np.array([(i, j, k) for i in range(q) for j in range(q) for k in range(q)])
    for ex in range(nelem[0]):
        for ey in range(nelem[1]):
            for ez in range(nelem[2]):
                pts = (ex + loc[:, 0]) * nb[1] * nb[2] + (ey + loc[:, 1]) * nb[2] + (ez + loc[:, 2])
                dofs = (3 * pts[:, None] + np.arange(3)).ravel()
                keys = (dofs[:, None].astype(np.int64) * ndof + dofs[None, :]).ravel()
                idx = np.searchsorted(keys_csr, keys)
                assert np.all(keys_csr[idx] == keys)
                np.add.at(counts, idx, 1.0)
    return counts


def formula_counts(nelem, rowptr, cols, p=2):
    """Closed form: the elements holding both control points, per direction."""
    nb = [n + p for n in nelem]
    ndof = 3 * nb[0] * nb[1] * nb[2]
    rowidx = np.repeat(np.arange(ndof), np.diff(rowptr))
    out = np.ones(len(cols))
    ci, cj = rowidx // 3, cols // 3
    strides = [nb[1] * nb[2], nb[2], 1]
    for d in range(3):
        i = (ci // strides[d]) % nb[d]
        j = (cj // strides[d]) % nb[d]
        lo = np.maximum(np.maximum(i, j) - p, 0)
        hi = np.minimum(np.minimum(i, j), nelem[d] - 1)
        out *= np.maximum(hi - lo + 1, 0)
    return out
