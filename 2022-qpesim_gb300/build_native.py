"""Builds the in-tree native library lib/libqpe_gb300.so for sm_103a.

Each translation unit under csrc/ is compiled by nvcc in parallel
(-gencode arch=compute_103a,code=sm_103a), then linked into one shared library
with a C ABI (include/qpe_gb300.h). Objects go to _build/ next to this file.
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
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libqpe_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build qpesim_gb300")


def sources() -> list[Path]:
    return sorted(p for p in CSRC.iterdir() if p.suffix in (".cu", ".cpp"))


def _compile(nvcc: str, src: Path, obj: Path, verbose: bool) -> None:
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles csrc/ into lib/libqpe_gb300.so unless it is newer than every source."""
    srcs = sources()
    headers = [p for p in CSRC.iterdir() if p.suffix in (".h", ".cuh")]
    headers += list((PKG.parent / "include").glob("*.h"))
    newest = max(p.stat().st_mtime for p in srcs + headers + [Path(__file__)])
    if not force and LIB.exists() and LIB.stat().st_mtime > newest and _is_native_arch(LIB):
        return LIB
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    objs = [BUILD / (s.stem + ("_cpp" if s.suffix == ".cpp" else "") + ".o") for s in srcs]
    workers = min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        futs = [ex.submit(_compile, nvcc, s, o, verbose) for s, o in zip(srcs, objs)]
        for f in futs:
            f.result()
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


def _is_native_arch(path: Path) -> bool:
    """True if the ELF machine of `path` matches this host (a library built on
    another architecture must be rebuilt here)."""
    import platform
    try:
        with open(path, "rb") as f:
            head = f.read(20)
        machine = int.from_bytes(head[18:20], "little")
    except OSError:
        return False
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    return want is None or machine == want


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
