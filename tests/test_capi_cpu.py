"""The C ABI library loads and exports every symbol include/afem_gb300.h
declares; argument validation works without a GPU."""
import ctypes as C
import os
import re

import pytest

from arcanefem_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "afem_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(afem_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def L():
    if not os.path.exists(_capi.LIB_PATH):
        from arcanefem_gb300 import build
        build.build()
    return _capi.lib()


def test_every_declared_symbol_is_exported(L):
    syms = header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert set(syms) == set(_capi.SIGNATURES), "binding and header disagree"


def test_version_and_errors_without_gpu(L):
    assert L.afem_version() == 10000
    # null output handle -> AFEM_ERR_BAD_ARG, message set, nothing touches the GPU
    assert L.afem_context_create(None, None) == 1
    assert b"null output" in L.afem_last_error()
    assert L.afem_ls_eliminate_row(None, 0, 0.0) == 1
    assert L.afem_node_cell_build(None, 1, 1, 3, None, None, None, None, None) == 1
    opt = _capi.SolverOptions()
    L.afem_solver_options_default(C.byref(opt))
    assert opt.rtol == 1e-7 and opt.max_iter == 1000 and opt.precond == _capi.PRECOND_JACOBI


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_capi, "_lib", None)
    monkeypatch.setattr(_capi, "LIB_PATH", str(tmp_path / "nope.so"))
    with pytest.raises(RuntimeError, match="no fallback"):
        _capi.lib()
