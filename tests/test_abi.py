"""The C-ABI boundary without a GPU: the library builds for sm_103a, loads, and
exports every function include/formoniq_gpu.h declares; no compute is called."""
import ctypes
import os
import re
import shutil
import subprocess

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


C_BASE = {"int": "c_int", "fq_status": "c_int", "fq_form": "c_int", "fq_bc": "c_int", "fq_precision": "c_int",
          "int32_t": "i32", "int64_t": "i64", "uint64_t": "u64", "int8_t": "i8", "double": "f64", "void": "c_void",
          "char": "c_char", "size_t": "usize"}


def c_to_rust(ctype):
    """A C parameter or return type in Rust FFI spelling: the base renamed
    (fq_x -> FqX, enums -> c_int), each pointer level *const or *mut by the
    constness of what it points to (const T* -> *const T; T* const* -> *const *mut T)."""
    toks = re.findall(r"const|\*|[A-Za-z_][A-Za-z0-9_]*", ctype)
    base_const, base, levels = False, None, []  # levels: constness of each pointer itself
    for t in toks:
        if t == "const":
            if base is None:
                base_const = True
            elif levels:
                levels[-1] = True
            else:
                base_const = True
        elif t == "*":
            levels.append(False)
        else:
            base = t
    name = C_BASE.get(base) or "".join(w.capitalize() for w in base.split("_"))
    pointee_const = [base_const] + levels[:-1]
    return "".join("*const " if c else "*mut " for c in reversed(pointee_const)) + name if levels else name


def header_prototypes():
    """name -> (return type, [parameter types]) in Rust spelling."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for ret, name, args in re.findall(r"([A-Za-z_][A-Za-z0-9_ \*]*?)\s*\b(fq_[a-z0-9_]+)\s*\(([^;{()]*)\)\s*;", text):
        ret = ret.split()[-2:] if ret.split()[-1:] == ["*"] else ret
        ret = " ".join(ret) if isinstance(ret, list) else ret
        params = [] if args.strip() in ("", "void") else [a.strip() for a in args.split(",")]
        ptypes = [c_to_rust(re.sub(r"\b[A-Za-z_][A-Za-z0-9_]*\s*$", "", a)) for a in params]
        rt = c_to_rust(ret.strip())
        out[name] = (None if rt == "c_void" else rt, ptypes)
    return out


def rust_prototypes():
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = "\n".join(re.findall(r"```rust\n(.*?)```", doc, flags=re.S))
    out = {}
    for name, args, ret in re.findall(r"\bfn (fq_[a-z0-9_]+)\s*\(([^)]*)\)\s*(?:->\s*([^;]+))?;", blocks):
        params = [a for a in (x.strip() for x in args.split(",")) if a]
        ptypes = [re.sub(r"\s+", " ", a.split(":", 1)[1].strip()).replace("c_double", "f64") for a in params]
        out[name] = (re.sub(r"\s+", " ", ret.strip()).replace("c_double", "f64") if ret else None, ptypes)
    return out


def header_struct_fields(name):
    """(field, type) of a header typedef struct, in order (comma lists split)."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    body = re.search(r"typedef struct " + name + r" \{(.*?)\} " + name + ";", text, flags=re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(.*?)([A-Za-z_][A-Za-z0-9_]*(?:\s*,\s*[A-Za-z_][A-Za-z0-9_]*)*)$", decl, flags=re.S)
        ctype, names = m.group(1), [x.strip() for x in m.group(2).split(",")]
        out += [(n, c_to_rust(ctype)) for n in names]
    return out


def test_rust_structs_mirror_the_header():
    """FqSolveOpts and FqReport in the binding have the header's fields, in
    order, with the header's types (repr(C) then lays them out alike)."""
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    for rust, c in (("FqSolveOpts", "fq_solve_opts"), ("FqReport", "fq_report")):
        body = re.search(r"pub struct " + rust + r" \{(.*?)\}", doc, flags=re.S).group(1)
        got = [(m.group(1), m.group(2).strip()) for m in re.finditer(r"pub (\w+): ([\w* ]+)", body)]
        want = header_struct_fields(c)
        assert got == want, (rust, got, want)


def test_c_types_spell_in_rust():
    assert c_to_rust("const fq_matrix* const* mats".rsplit(" ", 1)[0]) == "*const *const FqMatrix"
    assert c_to_rust("fq_matrix* const*") == "*const *mut FqMatrix"
    assert c_to_rust("const int32_t**") == "*mut *const i32"
    assert c_to_rust("fq_bc") == "c_int"
    assert c_to_rust("const fq_solve_opts*") == "*const FqSolveOpts"


def test_rust_binding_covers_the_header():
    """The extern blocks a formoniq maintainer adds bind every entry point with
    the header's parameter and return types (pointer mutability included)."""
    want, bound = header_prototypes(), rust_prototypes()
    assert sorted(want) == declared_functions()
    assert sorted(bound) == sorted(want), (sorted(set(want) - set(bound)), sorted(set(bound) - set(want)))
    wrong = {n: (bound[n], want[n]) for n in want if bound[n] != want[n]}
    assert not wrong, wrong


C_SCALAR = {"int": "i4", "fq_status": "i4", "fq_form": "i4", "fq_bc": "i4", "fq_precision": "i4", "int32_t": "i4",
            "int64_t": "i8", "uint64_t": "u8", "int8_t": "i1", "double": "f8", "char": "i1", "size_t": "u8"}
C_STRUCTS = {"fq_solve_opts": "SolveOpts", "fq_report": "_Report", "fq_request": "_Request", "fq_result": "_Result",
             "fq_server_stats": "_ServerStats"}


def c_kind(ctype):
    """A C type as a kind: scalars by class and width, pointers by pointee,
    the header's structs by their ctypes mirror, handles opaque."""
    toks = [t for t in re.findall(r"\*|[A-Za-z_][A-Za-z0-9_]*", ctype) if t != "const"]
    base = next(t for t in toks if t != "*")
    kind = C_SCALAR.get(base) or ("struct:" + C_STRUCTS[base] if base in C_STRUCTS else
                                  "void" if base == "void" else "opaque")
    for _ in range(toks.count("*")):
        kind = "ptr:" + kind
    return kind


def ctypes_kind(t):
    if t is None:
        return "void"
    if t is ctypes.c_void_p:
        return "ptr:any"
    if t is ctypes.c_char_p:
        return "ptr:i1"
    if issubclass(t, ctypes._Pointer):
        return "ptr:" + ctypes_kind(t._type_)
    if issubclass(t, ctypes.Structure):
        return "struct:" + t.__name__
    code = t._type_
    cls = "f" if code in "fd" else ("u" if code.isupper() else "i")
    return f"{cls}{ctypes.sizeof(t)}"


def kinds_match(c, py):
    if py == "ptr:any":
        return c.startswith("ptr:")
    if c.startswith("ptr:") and py.startswith("ptr:"):
        return kinds_match(c[4:], py[4:]) or (c[4:] == "opaque" and py[4:] == "any")
    return c == py


def header_c_prototypes():
    """name -> (return type, [parameter types]) as written in the header."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for ret, name, args in re.findall(r"([A-Za-z_][A-Za-z0-9_ \*]*?)\s*\b(fq_[a-z0-9_]+)\s*\(([^;{()]*)\)\s*;", text):
        params = [] if args.strip() in ("", "void") else [a.strip() for a in args.split(",")]
        out[name] = (ret.strip(), [re.sub(r"\b[A-Za-z_][A-Za-z0-9_]*\s*$", "", a) for a in params])
    return out


def test_ctypes_signatures_match_the_header():
    """Every ctypes argtype and restype of the binding has the header's class
    and width (c_void_p standing for any pointer): a wrong integer width here
    would pass truncated sizes to the device."""
    import formoniq_gb300 as fq

    want = header_c_prototypes()
    wrong = {}
    for name, (res, args) in fq._SIGNATURES.items():
        cret, cargs = want[name]
        if len(args) != len(cargs) or not kinds_match(c_kind(cret), ctypes_kind(res)) or not all(
                kinds_match(c_kind(c), ctypes_kind(a)) for c, a in zip(cargs, args)):
            wrong[name] = ([c_kind(c) for c in [cret] + cargs], [ctypes_kind(a) for a in [res] + args])
    assert not wrong, wrong


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the header's structs have its field offsets and
    sizes, as a C compiler lays them out (gcc on the header itself)."""
    import formoniq_gb300 as fq

    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "formoniq_gpu.h"', "int main(void) {"]
    for cname, pyname in C_STRUCTS.items():
        lines.append(f'printf("{cname} __size__ %zu\\n", sizeof({cname}));')
        for fname, _ in getattr(fq, pyname)._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines))
    subprocess.run([gcc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        struct, field, value = line.split()
        got[(struct, field)] = int(value)
    for cname, pyname in C_STRUCTS.items():
        cls = getattr(fq, pyname)
        assert got[(cname, "__size__")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)


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
