"""The C-ABI boundary without a GPU: the library builds for sm_103a, loads, and
exports every function include/formoniq_gpu.h declares; no compute is called."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "formoniq_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(fq_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def native():
    import formoniq_gb300 as fq
    from formoniq_gb300 import _build

    _build.build()
    return fq.load()


def test_header_declares_the_path():
    names = declared_functions()
    for must in ("fq_assemble", "fq_cell_metrics", "fq_element_matrices", "fq_minres", "fq_cg", "fq_solve_source",
                 "fq_solve_dirac_source", "fq_mixed_create", "fq_spmv"):
        assert must in names


def test_every_declared_symbol_is_exported(native):
    missing = [n for n in declared_functions() if not hasattr(native, n)]
    assert not missing, missing


def test_binding_covers_the_header():
    import formoniq_gb300 as fq

    assert sorted(fq.exported_symbols()) == declared_functions()


def header_arities():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for name, args in re.findall(r"\b(fq_[a-z0-9_]+)\s*\(([^;{()]*)\)\s*;", text):
        args = args.strip()
        out[name] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_rust_binding_covers_the_header():
    """The extern blocks a formoniq maintainer adds bind every entry point,
    each with the header's number of arguments."""
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = "\n".join(re.findall(r"```rust\n(.*?)```", doc, flags=re.S))
    bound = {}
    for name, args in re.findall(r"\bfn (fq_[a-z0-9_]+)\s*\(([^)]*)\)", blocks):
        args = args.strip().rstrip(",")
        bound[name] = 0 if not args else args.count(",") + 1
    want = header_arities()
    assert sorted(want) == declared_functions()
    assert sorted(bound) == sorted(want), (sorted(set(want) - set(bound)), sorted(set(bound) - set(want)))
    wrong = {n: (bound[n], want[n]) for n in want if bound[n] != want[n]}
    assert not wrong, wrong


def test_status_names(native):
    native.fq_status_name.restype = ctypes.c_char_p
    assert native.fq_status_name(0) == b"FQ_OK"
    assert native.fq_status_name(8) == b"FQ_NO_DEVICE"


def test_context_without_device_fails_loudly(native):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a device is present")
    import formoniq_gb300 as fq

    with pytest.raises(fq.FqError) as e:
        fq.Context(0)
    assert e.value.name == "FQ_NO_DEVICE"


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No CPU fallback: without the CUDA library every entry point raises."""
    import formoniq_gb300 as fq

    monkeypatch.setattr(fq, "_lib", None)
    monkeypatch.setattr(fq, "lib_path", lambda: str(tmp_path / "libformoniq_gb300.so"))
    with pytest.raises(fq.FqUnavailable):
        fq.load()
    with pytest.raises(fq.FqUnavailable):
        fq.Context(0)


def test_kernels_are_blackwell_native():
    """The hot kernels are built for sm_103a only (one -gencode)."""
    from formoniq_gb300 import _build

    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
