"""CPU checks of the C ABI library: it builds, loads, and exports every
function include/rsvdt.h declares; without a GPU, creating a context fails
cleanly with RSVDT_ERR_CUDA (no CPU fallback). No compute calls."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rsvdt.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rsvdt_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_documented_entry_points():
    names = declared_functions()
    for must in ["rsvdt_create", "rsvdt_set_operator", "rsvdt_set_weight", "rsvdt_set_sketch", "rsvdt_action",
                 "rsvdt_qr_all_freqs", "rsvdt_svd_all_freqs", "rsvdt_run", "rsvdt_get_results",
                 "rsvdt_last_error", "rsvdt_destroy"]:
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    import ctypes

    lib = ctypes.CDLL(built_lib)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(built_lib):
    import rsvdt

    assert sorted(rsvdt.EXPORTED) == declared_functions()
    rsvdt.load_library()


def test_params_defaults_follow_the_reference(built_lib):
    # SourceCode/ReadUserInput.c:109-130: k = 3, q = 0, Display = 2.
    import rsvdt

    p = rsvdt.default_params()
    assert (p.k, p.q, p.Display, p.precision) == (3, 0, 2, 0)


def test_struct_layout_matches_the_header(built_lib):
    import ctypes

    import rsvdt

    # int64 x3, double, int32 (+pad), double x2, int32 x2, double, int32 x2
    assert ctypes.sizeof(rsvdt.Params) == 80
    assert ctypes.sizeof(rsvdt.Grid) == 72


def test_create_without_gpu_fails_cleanly(built_lib):
    import torch

    import rsvdt

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(rsvdt.RsvdtError) as e:
        rsvdt.Context(rsvdt.default_params(k=2, Nw=8, w=0.1, dt=0.1, TransientLength=1.0))
    assert e.value.status == rsvdt.ERR_CUDA


def test_invalid_params_are_rejected_before_the_device(built_lib):
    import rsvdt

    for bad in [dict(k=0), dict(Nw=0), dict(w=0.0), dict(dt=-1.0), dict(DiscFlg=1, beta=-0.5)]:
        kw = dict(k=2, Nw=8, w=0.1, dt=0.1, TransientLength=1.0)
        kw.update(bad)
        with pytest.raises(rsvdt.RsvdtError) as e:
            rsvdt.Context(rsvdt.default_params(**kw))
        assert e.value.status == rsvdt.ERR_ARG, bad


def test_c_and_ctypes_struct_layouts_agree(built_lib, tmp_path):
    """sizeof and field offsets of every struct in include/rsvdt.h, from a C
    compiler, equal the ctypes mirrors the binding passes across the ABI."""
    import ctypes
    import subprocess

    import rsvdt

    structs = {"rsvdt_params": rsvdt.Params, "rsvdt_grid": rsvdt.Grid, "rsvdt_trans_params": rsvdt.TransParams,
               "rsvdt_trans_info": rsvdt.TransInfo}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "rsvdt.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_debug_build_compiles_and_identifies_itself(built_lib):
    """The bounds-checked build (-DRSVDT_DEBUG) compiles, exports the same
    symbols and reports itself; the release build reports 0."""
    import ctypes

    from rsvdt import build

    dbg = ctypes.CDLL(build.build_library(debug=True))
    rel = ctypes.CDLL(built_lib)
    assert dbg.rsvdt_debug_build() == 1 and rel.rsvdt_debug_build() == 0
    missing = [n for n in declared_functions() if not hasattr(dbg, n)]
    assert not missing, missing
