"""The Fortran bind(C) module (include/bromoc_gpu_mod.f90) against the C
header (include/bromoc_gpu.h): every interface names a declared entry point
and passes the same arguments in the same order with matching kinds, and
every derived type mirrors its struct field for field.  No Fortran compiler
is needed: both files are read as text.  Where a compiler is present
(gfortran), the module is also compiled."""
import re
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HDR = (ROOT / "include" / "bromoc_gpu.h").read_text()
F90 = (ROOT / "include" / "bromoc_gpu_mod.f90").read_text()

# C scalar type -> kind class
C_SCALAR = {"int32_t": "i32", "uint32_t": "i32", "int64_t": "i64", "uint64_t": "i64",
            "double": "f64", "float": "f32", "int8_t": "i8", "uint8_t": "u8", "int": "i32",
            "char": "i8"}
F_KIND = {"integer(c_int32_t)": "i32", "integer(c_int)": "i32", "integer(c_int64_t)": "i64",
          "real(c_double)": "f64", "real(c_float)": "f32", "integer(c_int8_t)": "i8",
          "character(kind=c_char)": "i8"}
OPAQUE = {"bromoc_ctx", "bromoc_batch", "bromoc_adj", "void"}


def _strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", "", s, flags=re.S)


def c_functions():
    body = _strip_c_comments(HDR)
    out = {}
    for m in re.finditer(r"(?:const\s+)?(\w+)\s*(\*?)\s*(bromoc_\w+)\s*\(([^)]*)\)\s*;", body):
        ret, star, name, args = m.groups()
        params = []
        for a in args.split(","):
            a = a.strip()
            if not a or a == "void":
                continue
            a = a.replace("const ", "")
            mm = re.match(r"(\w+)\s*(\**)\s*(\w+)$", a)
            assert mm, (name, a)
            base, stars, _ = mm.groups()
            if stars == "":
                params.append(C_SCALAR[base])
            elif stars == "*":
                params.append("ptr" if base in OPAQUE else "ref:" + C_SCALAR.get(base, base))
            else:
                params.append("ref:ptr")
        rkind = "ptr" if star else C_SCALAR[ret]
        out[name] = (rkind, params)
    return out


def c_structs():
    body = _strip_c_comments(HDR)
    out = {}
    for m in re.finditer(r"typedef struct (bromoc_\w+)\s*\{(.*?)\}\s*\1\s*;", body, re.S):
        name, fields = m.groups()
        fl = []
        for decl in fields.split(";"):
            decl = decl.strip().replace("const ", "")
            if not decl:
                continue
            base, names = re.match(r"(\w+)\s+(.*)$", decl, re.S).groups()
            for part in names.split(","):
                part = part.strip()
                kind = "ptr" if part.startswith("*") else C_SCALAR[base]
                field = part.lstrip("*").strip()
                if "[" in field:  # a fixed array: name[n] -> (name, kind x n)
                    field, n = field[:-1].split("[")
                    kind = f"{kind}x{int(n)}"
                fl.append((field, kind))
        out[name] = fl
    return out


def f_types():
    out = {}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)end type \1", F90, re.S):
        name, body = m.groups()
        fl = []
        for line in body.strip().splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            decl, names = line.split("::")
            decl = decl.strip()
            kind = "ptr" if decl == "type(c_ptr)" else F_KIND[decl]
            for n in names.split(","):
                n = n.strip()
                if "(" in n:  # a fixed array: name(n) -> (name, kind x n)
                    n, dim = n[:-1].split("(")
                    fl.append((n, f"{kind}x{int(dim)}"))
                else:
                    fl.append((n, kind))
        out[name] = fl
    return out


def f_interfaces():
    out = {}
    for m in re.finditer(r"function (\w+)\(([^)]*)\)\s*&?\s*bind\(C, name=\"(\w+)\"\)\s*"
                         r"result\((\w+)\)(.*?)end function", F90.replace("&\n", " "), re.S):
        fname, args, cname, res, body = m.groups()
        if not cname.startswith("bromoc_"):
            continue  # libc's strlen, used by bromoc_error_message
        decls = {}
        for line in body.splitlines():
            line = line.split("!")[0].strip()
            if "::" not in line or line.startswith("import"):
                continue
            spec, names = line.split("::")
            attrs = [a.strip() for a in spec.split(",")]
            base = attrs[0]
            value = "value" in attrs
            for n in names.split(","):
                n = n.strip().replace("(*)", "")
                if base == "type(c_ptr)":
                    k = "ptr" if value else "ref:ptr"
                elif base.startswith("type("):
                    k = "ref:" + base[5:-1]
                else:
                    k = F_KIND[base] if value else "ref:" + F_KIND[base]
                decls[n] = k
        params = [decls[a.strip()] for a in args.split(",") if a.strip()]
        out[cname] = (decls[res].replace("ref:", ""), params, fname)  # a result
    return out


def _compatible(ck, fk):
    if ck == fk:
        return True
    # an address passed as type(c_ptr), value serves any C pointer argument
    return fk == "ptr" and ck.startswith("ref:")


def test_interfaces_match_header():
    cf, fi = c_functions(), f_interfaces()
    assert len(fi) >= 40
    for cname, (fret, fparams, fname) in fi.items():
        assert fname == cname, (fname, cname)
        assert cname in cf, f"{cname} is not declared in bromoc_gpu.h"
        cret, cparams = cf[cname]
        assert cret == fret, (cname, cret, fret)
        assert len(cparams) == len(fparams), (cname, cparams, fparams)
        for k, (a, b) in enumerate(zip(cparams, fparams)):
            assert _compatible(a, b), (cname, k, a, b)


def test_hot_path_entry_points_bound():
    """The calls simul1 swaps in (energy, dynamics, interact, grand, the BD
    loop) and the deck-time setup all have a Fortran interface."""
    fi = f_interfaces()
    for name in ("create", "destroy", "last_error", "set_system", "set_types", "set_pairs",
                 "set_sites", "set_phix", "set_phiv", "set_rfpar", "set_membrane",
                 "set_diffusion", "set_countions", "set_buffers", "set_particles",
                 "get_particles", "energy", "interact", "dynamics", "bd_steps",
                 "bd_steps_host", "simul_cycles_host", "grand", "get_buffers",
                 "get_countions", "get_dids", "efpot_from_knots"):
        assert "bromoc_gpu_" + name in fi, name


def test_every_entry_point_bound():
    """The module binds every entry point the header declares."""
    missing = set(c_functions()) - set(f_interfaces())
    assert not missing, sorted(missing)


def test_types_match_structs():
    cs, ft = c_structs(), f_types()
    assert set(ft) == set(cs), (set(ft) ^ set(cs))
    for name, cfields in cs.items():
        assert ft[name] == cfields, (name, cfields, ft[name])


def test_checker_catches_a_mismatch(monkeypatch):
    """A planted mismatch (an argument's kind, a missing field) is caught."""
    bad = F90.replace("      integer(c_int32_t), value :: terms, qforces\n",
                      "      integer(c_int32_t), value :: terms\n"
                      "      real(c_double), value :: qforces\n", 1)
    assert bad != F90
    monkeypatch.setattr(sys.modules[__name__], "F90", bad)
    with pytest.raises(AssertionError):
        test_interfaces_match_header()
    monkeypatch.setattr(sys.modules[__name__], "F90", F90.replace("    real(c_double) :: rsphe\n", ""))
    with pytest.raises(AssertionError):
        test_types_match_structs()


@pytest.mark.skipif(shutil.which("gfortran") is None, reason="no Fortran compiler here")
def test_module_compiles(tmp_path):
    r = subprocess.run(["gfortran", "-c", "-std=f2008", str(ROOT / "include" / "bromoc_gpu_mod.f90"),
                        "-J", str(tmp_path), "-o", str(tmp_path / "m.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
