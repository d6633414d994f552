"""Shared helpers of the parity tests (oracle = FP64 CPU restatement)."""
import numpy as np


def lognormal(n, sigma, seed):
    return np.exp(np.random.default_rng(seed).normal(0.0, sigma, n))


def csr_rowscaled_close(rp, ci, va, orp, oci, ova, rtol=1e-12, noise=None):
    """Pattern bit-exact; every entry within rtol of its row maximum; and, on
    entries >= 1e-2 of the row maximum, within max(rtol, 10*noise) relative,
    where `noise` is the largest relative change of those entries when the
    oracle sums its quadrature points in reverse order (the rounding floor of
    the reference algorithm itself).  Smaller entries -- cancellations and
    orthogonality zeros -- are held to the row-scaled bound only."""
    assert np.array_equal(rp, orp), "rowptr differs"
    assert np.array_equal(ci, oci), "colind differs"
    rows = np.repeat(np.arange(len(orp) - 1), np.diff(orp))
    rowmax = np.zeros(len(orp) - 1)
    np.maximum.at(rowmax, rows, np.abs(ova))
    err = np.abs(va - ova)
    scale = rowmax[rows]
    assert np.all(err <= rtol * scale + 1e-300), "row-scaled error %g" % np.max(err / np.maximum(scale, 1e-300))
    big = np.abs(ova) >= 1e-2 * scale
    rel = err[big] / np.abs(ova[big])
    tol = rtol
    if noise is not None:
        n = np.abs(noise - ova)[big] / np.abs(ova[big])
        tol = max(rtol, 10 * float(n.max()))
    assert np.all(rel <= tol), "relative error %g (tolerance %g)" % (rel.max(), tol)


def permute_tets(elements, seed):
    """Random local vertex order per tet (all 24 orientation classes occur)."""
    rng = np.random.default_rng(seed)
    out = elements.copy()
    for e in range(len(out)):
        out[e] = out[e][rng.permutation(4)]
    return out
