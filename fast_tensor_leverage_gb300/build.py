"""Build recipe of libftl_gb300.so (the CUDA kernels behind the C ABI in
include/ftl.h).  Compiles every csrc/*.cu for sm_103a in parallel and links
one shared library in-tree at fast_tensor_leverage_gb300/_build/.

    python -m fast_tensor_leverage_gb300.build
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libftl_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-Xptxas",
    "-O3",
    "--expt-relaxed-constexpr",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libftl_gb300")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _needs_rebuild() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "ftl.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False, defines: list[str] | None = None,
          out: Path | None = None) -> Path:
    """Compile and link.  `defines` (e.g. ["FTL_DESC_PREFETCH=0"]) and `out`
    build a tuning variant of the library next to the default one."""
    lib_path = Path(out) if out is not None else LIB
    if not force and defines is None and out is None and not _needs_rebuild():
        return LIB
    build_dir = lib_path.parent / (lib_path.stem + "_obj") if out is not None else BUILD
    build_dir.mkdir(parents=True, exist_ok=True)
    extra = [f"-D{d}" for d in (defines or [])]
    cc = nvcc()
    objs = []

    def compile_one(src: Path) -> Path:
        obj = build_dir / (src.stem + ".o")
        cmd = [cc, *NVCC_FLAGS, *extra, "-I", str(PKG.parent / "include"), "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr, file=sys.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = build_dir / (lib_path.name + ".tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
