"""Builds the CUDA library ``_build/libshg_gb300.so`` (and the ``shg`` CLI) for sm_103a.

Every translation unit in ``csrc/`` is compiled in parallel with nvcc; host code is built
with -ffp-contract=off so the crystal set-up keeps the reference's float operation order
on x86 and Arm alike.

Two diagnostic variants build the same sources into their own folders (no CLI):

* ``check`` (``_build_check/libshg_gb300_check.so``): -DSHG_CHECK, device-side index checks
  that record a failure site instead of faulting (csrc/shg_check.cuh, shg_check_status);
* ``sanitize`` (``_build_san/libshg_gb300_san.so``): host code with
  -fsanitize=address,undefined; load it with the ASan runtime preloaded.

``python -m shg_focused_gaussian_beams_gb300.build [--force] [-v] [--variant check|sanitize]``
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libshg_gb300.so")
CLI = os.path.join(OUT, "shg")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          f"-I{os.path.join(HERE, '..', 'include')}"]


VARIANTS = {
    "": {"out": OUT, "lib": "libshg_gb300.so", "flags": [], "link": []},
    "check": {"out": os.path.join(HERE, "_build_check"), "lib": "libshg_gb300_check.so", "flags": ["-DSHG_CHECK"],
              "link": []},
    "sanitize": {"out": os.path.join(HERE, "_build_san"), "lib": "libshg_gb300_san.so",
                 "flags": ["-Xcompiler", "-fsanitize=address", "-Xcompiler", "-fsanitize=undefined",
                           "-Xcompiler", "-fno-omit-frame-pointer", "-Xcompiler", "-fno-sanitize-recover=undefined"],
                 "link": ["-Xcompiler", "-fsanitize=address", "-Xcompiler", "-fsanitize=undefined"]},
}


def variant_lib(variant: str = "") -> str:
    v = VARIANTS[variant]
    return os.path.join(v["out"], v["lib"])


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        [os.path.join(HERE, "..", "include", "shg.h"), __file__]


def _obj(src, out=OUT):
    return os.path.join(out, os.path.basename(src) + ".o")


def _compile(src, verbose=False, variant=""):
    v = VARIANTS[variant]
    flags = COMMON + v["flags"]
    obj = _obj(src, v["out"])
    cmd = [NVCC] + ARCH + flags + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC] + flags + ["-x", "cu", "-c", src, "-o", obj] + ARCH
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def up_to_date(variant: str = "") -> bool:
    targets = [variant_lib(variant)] + ([CLI] if variant == "" else [])
    if not all(os.path.isfile(t) for t in targets):
        return False
    t = min(os.path.getmtime(x) for x in targets)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, jobs: int = 8, verbose: bool = False, variant: str = "") -> str:
    v = VARIANTS[variant]
    lib = variant_lib(variant)
    if not force and up_to_date(variant):
        return lib
    os.makedirs(v["out"], exist_ok=True)
    srcs = [s for s in _sources() if not s.endswith("shg_cli.cpp")]
    units = srcs + ([os.path.join(CSRC, "shg_cli.cpp")] if variant == "" else [])
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, variant), units))
    if verbose:
        for _, err in results:
            sys.stderr.write(err)
    objs = [_obj(s, v["out"]) for s in srcs]
    tmp = lib + f".tmp{os.getpid()}"
    subprocess.run([NVCC] + ARCH + v["link"] + ["-shared", "-o", tmp] + objs + ["-lcudart", "-ldl"], check=True)
    os.replace(tmp, lib)
    if variant == "":
        tmp = CLI + f".tmp{os.getpid()}"
        subprocess.run([NVCC] + ARCH + ["-o", tmp, _obj(os.path.join(CSRC, "shg_cli.cpp"))] + objs + ["-ldl"],
                       check=True)
        os.replace(tmp, CLI)
    return lib


if __name__ == "__main__":
    var = sys.argv[sys.argv.index("--variant") + 1] if "--variant" in sys.argv else ""
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, variant=var))
