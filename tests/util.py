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


def assert_cg_history_close(hist, ref, rtol=1e-6, knee=1e-4, late_factor=4.0):
    """CG residual histories of two FP64 runs that differ only in rounding.
    They agree to `rtol` while the residual is above `knee` of the first one.
    Below that, the loss of orthogonality in the Krylov vectors amplifies
    rounding. On the oracle alone, a 2e-16 relative change of the matrix entries
    moves entries of the hex p=3 history by more than 1e-6 once the residual is
    below ~1e-5 of the first, and moves late entries by up to 25 %; the GPU's
    assembled matrices differ from run to run in the last bit (the order of the
    FP64 atomic additions) and have moved late tet p=2 entries by 58 %.  So from
    there on the entries are only held within a factor `late_factor` of each
    other (the iteration counts and the solutions are compared by the callers).
    The last two entries, where one run may already have stopped, are not
    compared."""
    hist, ref = np.asarray(hist), np.asarray(ref)
    k = min(len(hist), len(ref)) - 2
    assert k > 10, "histories too short to compare"
    early = ref[:k] >= knee * ref[0]
    rel = np.abs(hist[:k] - ref[:k]) / ref[:k]
    assert np.all(rel[early] <= rtol), "history differs by %g above the knee" % rel[early].max()
    ratio = hist[:k] / ref[:k]
    assert np.all((ratio <= late_factor) & (ratio >= 1.0 / late_factor)), \
        "history differs by a factor %g" % max(ratio.max(), 1.0 / ratio.min())
