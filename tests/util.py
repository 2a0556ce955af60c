import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def relerr(a, b):
    """max |a - b| relative to the largest magnitude of b (field-wise scale)."""
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    assert a.shape == b.shape, (a.shape, b.shape)
    if a.size == 0:
        return 0.0
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def elemrel(a, b, floor):
    """max over entries of |a - b| / max(|b|, floor): the per-element relative
    error, with an absolute floor (in b's units) below which an entry counts
    as that small.  Reported beside relerr, which scales every entry by the
    field's largest magnitude and so hides errors of small entries."""
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    assert a.shape == b.shape, (a.shape, b.shape)
    if a.size == 0:
        return 0.0
    return float((np.abs(a - b) / np.maximum(np.abs(b), floor)).max())


def pair_q(x, i, j, h):
    """q = |x_i - x_j| / h in FP64 with the reference's operation order
    (GLM's component-wise difference, (x*x + y*y) + z*z, sqrt, division)."""
    r = x[i] - x[j]
    r2 = r[:, 0] * r[:, 0] + r[:, 1] * r[:, 1] + r[:, 2] * r[:, 2]
    rl = np.sqrt(r2)
    return rl, rl / h


def csr_rows(off):
    return np.repeat(np.arange(len(off) - 1), np.diff(off))


def solver_lists(x, off, nbr, h):
    """From the reference's neighbour sets (every candidate with q <= 1,
    itself included, in walk order) the pairs its DFSPH sums carry a non-zero
    kernel gradient for (CubicSpline::gradW, CubicSpline.h:53-73):
    j != i, |r| > 1e-5, q < 1.  Returns (rows, nbr) of the kept pairs."""
    rows = csr_rows(off)
    rl, q = pair_q(x, rows, nbr, h)
    keep = (nbr != rows) & (rl > 1.0e-5) & (q < 1.0)
    return rows[keep], nbr[keep]


def compare_lists(x, h, ref_rows, ref_nbr, got_off, got_nbr, got_count, kmax, band):
    """Compare a dump of pair lists with the reference's solver lists, per
    particle and in order, leaving out on both sides the pairs whose FP64
    distance lies within `band` of h (|q - 1| <= band: there the FP32 form's
    rounding decides, at the 1e-7 level, which side of h a pair falls on).
    Particles whose list overflowed (count > kmax) are skipped.  Returns
    (mismatching particles, band pairs, pairs compared, overflowed)."""
    n = len(got_off) - 1
    got_rows = csr_rows(got_off)
    _, gq = pair_q(x, got_rows, got_nbr, h)
    _, rq = pair_q(x, ref_rows, ref_nbr, h)
    gk = np.abs(gq - 1.0) > band
    rk = np.abs(rq - 1.0) > band
    band_pairs = int((~gk).sum() + (~rk).sum())
    g_rows, g_nbr = got_rows[gk], got_nbr[gk]
    r_rows, r_nbr = ref_rows[rk], ref_nbr[rk]
    over = np.asarray(got_count[:n]) > kmax
    # sequences per particle: equal counts and equal entries in order
    gc = np.bincount(g_rows, minlength=n)
    rc = np.bincount(r_rows, minlength=n)
    bad = set(np.nonzero((gc != rc) & ~over)[0].tolist())
    ok = (gc == rc) & ~over
    gm = ok[g_rows]
    rm = ok[r_rows]
    diff = g_nbr[gm] != r_nbr[rm]
    bad |= set(g_rows[gm][diff].tolist())
    return sorted(bad), band_pairs, int(gm.sum()), int(over.sum())
