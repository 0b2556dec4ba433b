"""Golden cases: the reference's own test meshes and solution check files
(fixtures made by tests/golden/make_fixtures.py), with the parameters of the
.arc inputs they come from.  Shared by the oracle pinning tests (CPU) and the
end-to-end GPU tests."""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_fixtures import CASES  # noqa: E402

sys.path.pop(0)


def load(name: str) -> dict:
    return dict(np.load(os.path.join(HERE, "golden", name + ".npz")))


def compare(name: str, u: np.ndarray, data: dict) -> float:
    """Max relative error over the check file, as checkNodeResultFile
    (femutils/FemUtils.cc:85-171): uid -> node by gmsh tag, values whose
    magnitude is below min_value are skipped."""
    spec = CASES[name]
    tags = data["node_tags"]
    lid = {int(t): i for i, t in enumerate(tags)}
    idx = np.array([lid[int(u_)] for u_ in data["check_uid"]])
    ref = data["check_val"]
    got = u.reshape(len(tags), -1)[idx][:, : ref.shape[1]]
    mask = np.abs(ref) > spec["min_value"]
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
    return float(err[mask].max())


def scalar_csr_from_block(rp: np.ndarray, cols: np.ndarray, b: int):
    """Scalar CSR structure of a b x b BSR whose values use the per-row layout
    (what BSRMatrix::toCsr produces, femutils/BSRFormat.cc:110-172)."""
    n = rp.size - 1
    lens = np.diff(rp)
    srp = np.zeros(n * b + 1, np.int64)
    srp[1:] = np.cumsum(np.repeat(lens * b, b))
    parts = []
    for i in range(n):
        blk = cols[rp[i]:rp[i + 1]]
        row = (b * np.repeat(blk, b) + np.tile(np.arange(b), blk.size))
        parts.extend([row] * b)
    scols = np.concatenate(parts).astype(np.int32)
    return srp.astype(np.int32), scols
