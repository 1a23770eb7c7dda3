"""The C ABI library: builds, loads, exports every symbol the header declares, and refuses
to run without a GPU (no CPU fallback).  No GPU needed."""
import os
import re

import pytest

from tests.conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from cudaprob3_gb300 import _abi, build
    build.build()
    return _abi.lib()


def header_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            syms |= set(re.findall(r"\b(cp3_[a-z0-9_]+)\s*\(", text))
    return syms


def test_header_and_binding_agree():
    from cudaprob3_gb300 import _abi
    assert header_symbols() == set(_abi.EXPORTS)


def test_library_exports_every_header_symbol(lib):
    for name in header_symbols():
        assert hasattr(lib, name), name


def test_library_targets_sm103a():
    from cudaprob3_gb300 import build
    src = open(build.__file__).read()
    assert "arch=compute_103a,code=sm_103a" in src


def test_create_without_gpu_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from cudaprob3_gb300 import AtmosCudaPropagatorSingle
    from cudaprob3_gb300._abi import CP3Error
    with pytest.raises(CP3Error, match="No GPU found"):
        AtmosCudaPropagatorSingle(0, 4, 4)


def test_null_handle_is_an_error(lib):
    import ctypes as C
    rc = lib.cp3_set_mns(None, 0.1, 0.1, 0.1, 0.0, 1)
    assert rc != 0
    assert b"null" in lib.cp3_last_error(None)


def test_build_is_stale_when_unit_flags_change(monkeypatch):
    """The library is rebuilt when a compile command changes, not only when a source does:
    cp3_tables.cu's -fmad=false is what the FP64 parity rests on."""
    from cudaprob3_gb300 import build
    base = build._signature("nvcc", ["-O3"], False)
    assert build._signature("nvcc", ["-O3"], False) == base
    monkeypatch.setattr(build, "UNITS", [(u, [] if u == "cp3_tables.cu" else f)
                                         for u, f in build.UNITS])
    assert build._signature("nvcc", ["-O3"], False) != base
    monkeypatch.undo()
    monkeypatch.setattr(build, "ARCH", ["-gencode", "arch=compute_100a,code=sm_100a"])
    assert build._signature("nvcc", ["-O3"], False) != base
    monkeypatch.undo()
    assert build._signature("nvcc", ["-O3"], True) != base


def test_reference_tree_comes_from_the_environment(monkeypatch, tmp_path):
    from oracle import oracle
    (tmp_path / "physics.hpp").write_text("// stand-in\n")
    monkeypatch.setenv("CP3_REFERENCE_DIR", str(tmp_path))
    assert oracle.reference_dir() == str(tmp_path)
    monkeypatch.setenv("CP3_REFERENCE_DIR", str(tmp_path / "absent"))
    got = oracle.reference_dir()  # falls back to the untracked copy, if there is one
    assert got is None or os.path.isfile(os.path.join(got, "physics.hpp"))
