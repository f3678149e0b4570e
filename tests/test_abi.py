"""The C-ABI library loads (no GPU needed) and exports every entry point that
include/bromoc_gpu.h declares; host-only entry points behave as documented."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

from bromoc_gb300 import abi

HEADER = Path(__file__).resolve().parents[1] / "include" / "bromoc_gpu.h"


def declared():
    txt = HEADER.read_text()
    return sorted(set(re.findall(r"\b(bromoc_gpu_\w+)\s*\(", txt)))


def test_header_lists_entry_points():
    names = declared()
    for n in ("bromoc_gpu_create", "bromoc_gpu_energy", "bromoc_gpu_interact",
              "bromoc_gpu_bd_steps", "bromoc_gpu_grand", "bromoc_gpu_dynamics"):
        assert n in names


def test_library_exports_every_symbol(gpu_lib):
    lib = gpu_lib.load()
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.bromoc_gpu_abi_version() == 2


def test_null_arguments_rejected(gpu_lib):
    lib = gpu_lib.load()
    assert lib.bromoc_gpu_create(0, 0, None, None) == abi.E_ARG
    h = C.c_void_p()
    assert lib.bromoc_gpu_create(-5, 0, None, C.byref(h)) == abi.E_ARG
    assert lib.bromoc_gpu_create(100, 7, None, C.byref(h)) == abi.E_ARG
    assert lib.bromoc_gpu_energy(None, 0, 0, None, None, None, None, None) == abi.E_ARG
    assert lib.bromoc_gpu_destroy(None) == abi.OK
    assert lib.bromoc_gpu_last_error(None) == b"null context"


def test_struct_layouts_match_header():
    """ctypes mirrors have the sizes the C compiler gives the structs."""
    src = HEADER.read_text()
    for cls, name in ((abi.System, "bromoc_system"), (abi.Types, "bromoc_types"),
                      (abi.Pairs, "bromoc_pairs"), (abi.Grid, "bromoc_grid"),
                      (abi.Membrane, "bromoc_membrane"),
                      (abi.Diffusion, "bromoc_diffusion"),
                      (abi.Buffers, "bromoc_buffers"),
                      (abi.PhivOpts, "bromoc_phiv_opts"),
                      (abi.Sites, "bromoc_sites")):
        m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, re.S)
        assert m, name
        body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            typ, rest = re.match(r"(const\s+)?(\w+)\s*(.*)", decl).group(2, 3)
            for v in rest.split(","):
                fields.append(v.strip().lstrip("*").strip())
        assert [f[0] for f in cls._fields_] == fields, name


def test_efpot_builder_rejects_bad_input(gpu_lib):
    with np.testing.assert_raises(abi.BromocError):
        gpu_lib.efpot_from_knots(np.array([0.0, 1.0, 2.0]),
                                 np.array([1.0, 2.0, 3.0]), 0.0, 0)
