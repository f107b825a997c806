"""Builds libsatgb.so in-tree with nvcc for sm_103a.

Every translation unit under csrc/ is compiled in parallel (one -gencode,
-lineinfo, -O3) and linked into ``sat_gb300/_lib/libsatgb.so`` together with
the CUDA runtime.  Nothing is installed into site-packages: the library is
loaded from this directory by ``sat_gb300._lib``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libsatgb.so"
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

SOURCES = [
    "satgb_api.cu",
    "sat_inst_u8.cu",
    "sat_inst_i8.cu",
    "sat_inst_int32.cu",
    "sat_inst_f32.cu",
    "sat_inst_f64.cu",
    "box_filter.cu",
    "scan_rows_t.cu",
    "satgb_noalloc.cu",
    "batch_repack.cu",
]


def nvcc_path() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return os.path.join(home, "bin", "nvcc")


def lib_path() -> str:
    return os.path.join(OUT_DIR, LIB_NAME)


def _stale(target: str, deps) -> bool:
    if not os.path.isfile(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, jobs: int = 0) -> str:
    nvcc = nvcc_path()
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "satgb.h"))
    common = [nvcc, GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
              "-I", os.path.join(os.path.dirname(HERE), "include")]
    srcs = [s for s in SOURCES if os.path.isfile(os.path.join(CSRC, s))]
    objs = []
    cmds = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmds.append(common + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return r

    if cmds:
        n = jobs or min(len(cmds), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(run, cmds))
    target = lib_path()
    if force or cmds or _stale(target, objs):
        tmp = target + ".tmp"
        run([nvcc, GENCODE, "-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, target)
    # the reference's command line (sat A S D0 D1 R) over the library
    cli_src = os.path.join(CSRC, "sat_cli.cpp")
    cli = cli_path()
    if os.path.isfile(cli_src) and (force or _stale(cli, [cli_src, target])):
        run([nvcc, "-O2", "-std=c++17", "-I", os.path.join(os.path.dirname(HERE), "include"), "-o", cli + ".tmp",
             cli_src, "-L", OUT_DIR, "-lsatgb", "-lcudart", "-Xlinker", "-rpath,$ORIGIN"])
        os.replace(cli + ".tmp", cli)
    return target


def cli_path() -> str:
    return os.path.join(OUT_DIR, "sat")


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
