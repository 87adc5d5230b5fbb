"""The C-ABI library loads without a GPU and exports every entry point of include/shg.h."""
import os
import re

import pytest

from _util import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "shg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(shg_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_entry_points():
    names = _declared()
    assert "shg_run" in names and "shg_batch_run" in names and len(names) >= 15


def test_library_exports_all_declared_symbols():
    from shg_focused_gaussian_beams_gb300 import _lib
    L = _lib.lib()
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing
    # the Python binding covers every declared symbol
    assert set(_declared()) <= set(_lib.SIGNATURES), set(_declared()) - set(_lib.SIGNATURES)


def test_config_defaults_are_the_reference_constants():
    """SHG.cpp:11-13 and Crystal.h:31-53 (no CUDA call involved)."""
    from shg_focused_gaussian_beams_gb300 import _lib
    c = _lib.default_config()
    assert (c.nx, c.ny, c.nz) == (64, 64, 200)
    assert (c.lx, c.ly, c.lz) == (2000.0, 1000.0, 30000.0)
    import numpy as np
    f = np.float32
    assert f(c.deff) == f(11.00e-6) and f(c.lambda_qpm) == f(7.97) and f(c.alpha_p) == f(0.17e-6)
    assert f(c.alpha_s) == f(1.57e-6) and f(c.beta_s) == f(5e-5) and f(c.kth) == f(8.4e-6)
    assert f(c.htc) == f(10e-12) and c.thermal == 0 and c.sh_seed < 0


def test_invalid_arguments_fail_loudly_without_gpu():
    from shg_focused_gaussian_beams_gb300 import _lib
    import ctypes as C
    L = _lib.lib()
    assert L.shg_config_init(None) == 1
    assert L.shg_create(None, None) == 1
    assert L.shg_batch_create(None, None, 0, None) == 1
    assert b"null" in L.shg_last_error()


def test_python_sellmeier_matches_oracle():
    import numpy as np
    import oracle as O
    from shg_focused_gaussian_beams_gb300.workloads import sellmeier_n
    for T in np.linspace(10, 90, 41, dtype=np.float32):
        for L in (1.064, np.float32(0.532), 0.8):
            assert sellmeier_n(L, T) == O.lib().oracle_n_f32(L, T)


def test_check_status_of_a_build_without_checks():
    """The normal library reports that it carries no device-side checks, without a GPU."""
    import ctypes as C
    from shg_focused_gaussian_beams_gb300 import _lib
    L = _lib.lib()
    e, s, v = C.c_int(-1), C.c_int(-1), C.c_longlong(-1)
    assert L.shg_check_status(C.byref(e), C.byref(s), C.byref(v)) == 0
    assert (e.value, s.value, v.value) == (0, 0, 0)
    assert L.shg_check_status(None, C.byref(s), C.byref(v)) == 1
    assert L.shg_check_selftest(7) == 2 and b"SHG_CHECK" in L.shg_last_error()


def _header_struct_fields(name):
    """Field names of `typedef struct <name> {...}` in include/shg.h, in declaration order."""
    src = open(os.path.join(ROOT, "include", "shg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\}" % name, src, flags=re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        names = decl.split(None, 1)[1]  # drop the type
        out += [re.sub(r"\[.*\]", "", n).strip() for n in names.split(",")]
    return out


@pytest.mark.parametrize("cname,pyname", [("shg_config", "Config"), ("shg_instance", "Instance"),
                                          ("shg_kernel_stat", "KernelStat")])
def test_python_structs_match_the_header_layout(cname, pyname, tmp_path):
    """The ctypes structures of the binding have the header's fields, offsets and size (the
    offsets as the C compiler lays them out), so shg_config_init and the batch calls write
    exactly the Python objects' memory."""
    import ctypes as C
    import shutil
    import subprocess
    from shg_focused_gaussian_beams_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = _header_struct_fields(cname)
    py = getattr(_lib, pyname)
    assert [f[0] for f in py._fields_] == fields
    prog = ["#include <stddef.h>", "#include <stdio.h>", '#include "shg.h"', "int main(void) {",
            '  printf("%%zu\\n", sizeof(%s));' % cname]
    prog += ['  printf("%%zu\\n", offsetof(%s, %s));' % (cname, f) for f in fields]
    prog += ["  return 0;", "}"]
    c_src = tmp_path / "layout.c"
    c_src.write_text("\n".join(prog) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(c_src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert vals[0] == C.sizeof(py)
    assert vals[1:] == [getattr(py, f).offset for f in fields]


def _prototypes():
    """{name: (return type, [parameter types])} of every prototype in include/shg.h."""
    src = open(os.path.join(ROOT, "include", "shg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for ret, name, params in re.findall(r"^\s*((?:const\s+)?\w+(?:\s+\w+)?\s*\**)\s*(shg_\w+)\s*\(([^)]*)\)\s*;",
                                        src, flags=re.M):
        types = []
        for p in params.split(","):
            p = " ".join(p.split())
            if p in ("", "void"):
                continue
            types.append(re.sub(r"\s*\b\w+$", "", p))  # drop the parameter's name
        out[name] = (ret.strip(), types)
    return out


def test_binding_signatures_match_the_header_prototypes():
    """Every argtypes / restype of the ctypes binding agrees with the C prototype: the same
    number of arguments, the exact type of every scalar, and a pointer of the right kind for
    every pointer (a wrong count or width would corrupt the call silently)."""
    import ctypes as C
    from shg_focused_gaussian_beams_gb300 import _lib
    scalars = {"int": C.c_int, "float": C.c_float, "double": C.c_double, "long long": C.c_longlong}
    structs = {"shg_config": _lib.Config, "shg_instance": _lib.Instance, "shg_kernel_stat": _lib.KernelStat}
    opaque = {"void", "shg_handle", "shg_batch", "shg_thgrad"}

    def ok(ctype, bound):
        stars = ctype.count("*")
        base = " ".join(ctype.replace("const", " ").replace("*", " ").split())
        if stars == 0:
            return bound is scalars.get(base, object())
        if stars == 2:
            return bound is C.POINTER(C.c_void_p)
        if base == "char":
            return bound is C.c_char_p
        if base in scalars:
            return bound in (C.POINTER(scalars[base]), C.c_void_p)
        if base in structs:
            return bound is C.POINTER(structs[base])
        return base in opaque and bound is C.c_void_p

    protos = _prototypes()
    assert set(protos) == set(_declared())
    bad = []
    for name, (ret, params) in protos.items():
        res, args = _lib.SIGNATURES[name]
        want_res = {"int": C.c_int, "void": None, "double": C.c_double, "const char *": C.c_char_p}[ret]
        if res is not want_res or len(args) != len(params):
            bad.append((name, ret, params))
            continue
        bad += [(name, i, p) for i, (p, a) in enumerate(zip(params, args)) if not ok(p, a)]
    assert not bad, bad


def test_argument_errors_are_reported_before_any_device_call():
    """Grids the device path does not take, unknown crystals, empty batches and null
    arguments return their status codes and messages from host checks alone (this runs
    without a GPU)."""
    import ctypes as C
    from shg_focused_gaussian_beams_gb300 import _lib
    L = _lib.lib()
    h = C.c_void_p()
    for over, code, msg in [(dict(nx=48, ny=48), 2, b"power of two"), (dict(nx=64, ny=32), 2, b"square grid"),
                            (dict(nx=512, ny=512), 2, b"[16, 256]"), (dict(nz=1), 1, b"grid sizes")]:
        cfg = _lib.default_config(**over)
        assert L.shg_create(C.byref(cfg), C.byref(h)) == code and msg in L.shg_last_error(), over
    n = C.c_float()
    assert L.shg_index(7, 1.064, 50.0, C.byref(n)) == 1 and b"unknown crystal" in L.shg_last_error()
    assert L.shg_index(0, -1.0, 50.0, C.byref(n)) == 1
    assert L.shg_index(1, 1.064, 50.0, C.byref(n)) == 0 and 2.1 < n.value < 2.2
    cfg = _lib.default_config()
    assert L.shg_batch_create(C.byref(cfg), None, 0, C.byref(h)) == 1 and b"empty batch" in L.shg_last_error()
    assert L.shg_thgrad_create(C.byref(cfg), 0, C.byref(h)) == 2 and b"count" in L.shg_last_error()
    assert L.shg_dft2d_device(48, -1, None, None, None) == 1
    assert L.shg_dft2d_device(64, 0, None, None, None) == 1
    assert L.shg_run(None, 1, 1, 1, 1, 1, 1, 1, 1, 0) == 1 and b"null handle" in L.shg_last_error()
    assert L.shg_cwes_noalloc(None, 50.0, None, None, None, None, None, None) == 1
    assert L.shg_init_temperature(None, 50, 50, 50, 0, None) == 1 and b"null config" in L.shg_last_error()
    assert L.shg_heat_sweeps(None, None, None, 25.0, 1, 0) == 1 and b"null config" in L.shg_last_error()
    assert L.shg_destroy(None) == 0 and L.shg_batch_destroy(None) == 0
