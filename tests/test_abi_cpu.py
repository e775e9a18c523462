"""The C ABI as include/hpdex_gb300.h declares it, against the ctypes binding (CPU only).

A caller binds the library from the header alone (ctypes, cgo, JNI, a C or C++ host), so the
header and hpdex_gb300/_lib.py must agree on every detail that is not checked at call time:
- the header compiles as C99 and as C++17, warnings as errors;
- every constant the Python layer hard-codes (status codes, dtype codes, the zero_handling /
  alternative / method / exact_variant values, the plan modes) equals the header's value, as
  printed by a C program built against the header;
- hpdex_mwu_options has the layout of the ctypes structure: size and every field offset;
- every declared function has the ctypes signature the header implies: return type, number
  of parameters, and per parameter the integer width and signedness, double or float, and for
  pointers the pointee type wherever the binding names one;
- the ctypes stub a maintainer of the reference would add (hpdex_gb300/backend/bin/
  ctypes_stub.py) runs against the built library, binds hpdex_mannwhitneyu with the declared
  argument types and reports its errors (no GPU is needed: the library refuses before it reads
  any array); the C example (include/hpdex_gb300_example.c) compiles against the header.
"""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "hpdex_gb300.h")

SCALARS = {
    "int": ctypes.c_int,
    "int32_t": ctypes.c_int32,
    "int64_t": ctypes.c_int64,
    "uint64_t": ctypes.c_uint64,
    "double": ctypes.c_double,
    "float": ctypes.c_float,
}


def _header_text():
    with open(HEADER) as f:
        return re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)


def _declarations():
    """(return type, name, [parameter declarations]) for every function in the header."""
    out = []
    pat = re.compile(r"^(int|void|const char\s*\*)\s*(hpdex_\w+)\s*\(([^)]*)\)\s*;", re.M | re.S)
    for m in pat.finditer(_header_text()):
        params = [" ".join(p.split()) for p in m.group(3).split(",")]
        if params == ["void"]:
            params = []
        out.append((" ".join(m.group(1).split()), m.group(2), params))
    return out


def _integer_macros():
    return re.findall(r"^#define\s+(HPDEX_[A-Z0-9_]+)\s+(\S.*)$", _header_text(), flags=re.M)


def _compiler(name):
    path = shutil.which(name)
    if path is None:
        pytest.skip(f"{name} is not installed")
    return path


@pytest.mark.parametrize("lang,std,compiler", [("c", "-std=c99", "gcc"), ("c++", "-std=c++17", "g++")])
def test_header_compiles_cleanly(tmp_path, lang, std, compiler):
    cc = _compiler(compiler)
    src = tmp_path / ("use." + ("c" if lang == "c" else "cpp"))
    src.write_text('#include "hpdex_gb300.h"\nint main(void) { hpdex_mwu_options o; '
                   'hpdex_mwu_options_default(&o); return o.method == HPDEX_ASYMPTOTIC ? 0 : 1; }\n')
    r = subprocess.run([cc, std, "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only",
                        "-I", os.path.dirname(HEADER), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.fixture(scope="module")
def header_values(tmp_path_factory):
    """Every integer macro of the header and the options struct's layout, as C sees them."""
    cc = _compiler("gcc")
    d = tmp_path_factory.mktemp("abi")
    names = [n for n, v in _integer_macros() if not n.endswith("_H")]
    fields = re.search(r"typedef struct hpdex_mwu_options \{(.*?)\}", _header_text(), re.S).group(1)
    fields = re.findall(r"int32_t\s+(\w+)\s*;", fields)
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "hpdex_gb300.h"',
             "int main(void) {"]
    lines += [f'  printf("%s %lld\\n", "{n}", (long long)({n}));' for n in names]
    lines += ['  printf("sizeof %lld\\n", (long long)sizeof(hpdex_mwu_options));']
    lines += [f'  printf("offsetof.{f} %lld\\n", (long long)offsetof(hpdex_mwu_options, {f}));'
              for f in fields]
    lines += ["  return 0;", "}"]
    (d / "values.c").write_text("\n".join(lines) + "\n")
    exe = d / "values"
    subprocess.run([cc, "-std=c99", "-I", os.path.dirname(HEADER), str(d / "values.c"), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    vals = dict(line.split() for line in out.splitlines())
    return {k: int(v) for k, v in vals.items()}, fields


def test_python_constants_equal_the_header(header_values):
    from hpdex_gb300 import _lib, resident
    v, _ = header_values
    status = {"HPDEX_OK": _lib.HPDEX_OK, "HPDEX_ERR_RUNTIME": _lib.HPDEX_ERR_RUNTIME,
              "HPDEX_ERR_ARGUMENT": _lib.HPDEX_ERR_ARGUMENT, "HPDEX_ERR_CUDA": _lib.HPDEX_ERR_CUDA,
              "HPDEX_ERR_UNSUPPORTED": _lib.HPDEX_ERR_UNSUPPORTED,
              "HPDEX_ERR_TIMEOUT": _lib.HPDEX_ERR_TIMEOUT}
    for name, py in status.items():
        assert v[name] == py, name
    for dt, code in _lib.DTYPE_CODES.items():
        assert v["HPDEX_" + dt.upper()] == code, dt
    zh = {"none": "HPDEX_ZERO_NONE", "min": "HPDEX_ZERO_MIN", "max": "HPDEX_ZERO_MAX",
          "mix": "HPDEX_ZERO_MIX"}
    for k, name in zh.items():
        assert resident._ZH[k] == v[name], k
    alt = {"less": "HPDEX_LESS", "greater": "HPDEX_GREATER", "two-sided": "HPDEX_TWO_SIDED"}
    for k, name in alt.items():
        assert resident._ALT[k] == v[name], k
    assert resident._METHOD == {"exact": v["HPDEX_EXACT"], "asymptotic": v["HPDEX_ASYMPTOTIC"]}
    o = resident.make_options(exact_variant="reference")
    assert o.exact_variant == v["HPDEX_EXACT_REFERENCE"]
    o = resident.make_options(exact_variant="mwu_null")
    assert o.exact_variant == v["HPDEX_EXACT_MWU_NULL"]
    assert (resident.BATCHED, resident.PLAIN) == (v["HPDEX_MODE_BATCHED"], v["HPDEX_MODE_PLAIN"])


def test_options_struct_layout(header_values):
    from hpdex_gb300 import _lib
    v, fields = header_values
    assert [f for f, _ in _lib.MwuOptions._fields_] == fields
    assert ctypes.sizeof(_lib.MwuOptions) == v["sizeof"]
    for f in fields:
        assert getattr(_lib.MwuOptions, f).offset == v["offsetof." + f], f


def _expected_return(ret):
    return {"int": ctypes.c_int, "void": None, "const char*": ctypes.c_char_p}[ret]


def _check_param(decl, ct, MwuOptions):
    """One parameter declaration against its ctypes type; returns an error text or None."""
    typ = decl.rsplit(" ", 1)[0] if " " in decl else decl
    typ = typ.replace("const ", "").replace(" *", "*")
    stars = decl.count("*")
    base = typ.replace("*", "").strip()
    if stars == 0:
        want = SCALARS.get(base)
        if want is None:
            return f"no scalar mapping for {decl!r}"
        return None if ct is want else f"{decl!r}: {ct.__name__} instead of {want.__name__}"
    if ct in (ctypes.c_void_p, ctypes.c_char_p):
        return None  # an address: accepted for any pointer
    if not (isinstance(ct, type) and issubclass(ct, ctypes._Pointer)):
        return f"{decl!r}: {getattr(ct, '__name__', ct)} is not a pointer type"
    pointee = ct._type_
    if stars == 2:  # handle out-parameters (hpdex_matrix**, void**)
        return None if pointee is ctypes.c_void_p else f"{decl!r}: POINTER({pointee.__name__})"
    if base == "hpdex_mwu_options":
        return None if pointee is MwuOptions else f"{decl!r}: POINTER({pointee.__name__})"
    want = SCALARS.get(base)
    if want is None:
        return f"{decl!r}: opaque pointer bound as POINTER({pointee.__name__})"
    return None if pointee is want else f"{decl!r}: POINTER({pointee.__name__})"


def test_every_function_signature_matches_the_binding():
    from hpdex_gb300 import _lib
    decls = _declarations()
    assert len(decls) >= 30
    assert {n for _, n, _ in decls} == set(_lib.EXPORTS)
    errors = []
    for ret, name, params in decls:
        res, args = _lib.EXPORTS[name]
        if res is not _expected_return(ret):
            errors.append(f"{name}: returns {ret}, bound as {res}")
        if len(args) != len(params):
            errors.append(f"{name}: {len(params)} parameters, bound with {len(args)}")
            continue
        for decl, ct in zip(params, args):
            e = _check_param(decl, ct, _lib.MwuOptions)
            if e:
                errors.append(f"{name}: {e}")
    assert not errors, "\n".join(errors)


def test_signature_comparison_catches_a_planted_mismatch():
    """The signature comparison fails on a binding with a narrowed parameter."""
    from hpdex_gb300 import _lib
    assert _check_param("int64_t n_rows", ctypes.c_int32, _lib.MwuOptions) is not None
    assert _check_param("const int32_t* group_id", ctypes.POINTER(ctypes.c_int64),
                        _lib.MwuOptions) is not None
    assert _check_param("double clip", ctypes.c_float, _lib.MwuOptions) is not None
    assert _check_param("hpdex_matrix** out", ctypes.POINTER(ctypes.c_int64),
                        _lib.MwuOptions) is not None
    assert _check_param("const int64_t* indptr", ctypes.c_void_p, _lib.MwuOptions) is None


def test_integration_stub_binds_the_library_as_declared():
    import numpy as np
    from hpdex_gb300 import _lib
    from hpdex_gb300.backend.bin import ctypes_stub
    lib, mannwhitneyu = ctypes_stub.bind(_lib.lib_path())
    args = lib.hpdex_mannwhitneyu.argtypes
    want = _lib.EXPORTS["hpdex_mannwhitneyu"][1]
    assert len(args) == len(want)
    for a, w in zip(args, want):
        if isinstance(w, type) and issubclass(w, ctypes._Pointer):
            assert issubclass(a, ctypes._Pointer) and a._type_._fields_ == w._type_._fields_
        else:
            assert a is w
    with pytest.raises(RuntimeError, match="Unsupported dtype for data"):
        mannwhitneyu(np.ones(4, np.float16), np.arange(4), np.array([0, 4]),
                     np.zeros(4, np.int32), 1)
    if _lib.device_count() == 0:
        with pytest.raises(RuntimeError, match="no CUDA device"):
            mannwhitneyu(np.ones(4, np.float32), np.arange(4), np.array([0, 4]),
                         np.zeros(4, np.int32), 1)


def test_c_example_compiles_against_the_header():
    """include/hpdex_gb300_example.c compiles against the header as C99, warnings as errors."""
    src = os.path.join(ROOT, "include", "hpdex_gb300_example.c")
    cc = _compiler("gcc")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                        os.path.dirname(HEADER), src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
