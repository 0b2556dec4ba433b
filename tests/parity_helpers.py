"""Comparison helpers shared by the GPU parity tests (test infrastructure)."""
import numpy as np

REL = 1e-12


def rel_err_rows(got, ref, rp, b=1):
    """Max over entries of |got - ref| / max(|ref|, 1e-3 * max|row|); an
    all-zero row (a node in no cell) is compared absolutely."""
    ref = np.asarray(ref)
    got = np.asarray(got)
    row_of = np.repeat(np.arange(rp.size - 1), np.diff(rp) * b * b)
    rowmax = np.zeros(rp.size - 1)
    np.maximum.at(rowmax, row_of, np.abs(ref))
    denom = np.maximum(np.abs(ref), 1e-3 * rowmax[row_of])
    return float(np.max(np.abs(got - ref) / np.where(denom > 0, denom, 1.0)))


def assert_bit_exact(got, ref, what=""):
    """Every entry equal (np.array_equal; -0.0 == 0.0)."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    if not np.array_equal(got, ref):
        d = np.abs(got - ref)
        k = int(np.argmax(d))
        raise AssertionError(f"{what}: {int((got != ref).sum())} of {got.size} entries differ; "
                             f"largest at {k}: {got[k]!r} vs {ref[k]!r}")
