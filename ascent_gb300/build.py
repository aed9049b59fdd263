"""Build the renderer's native library, ``ascent_gb300/_lib/libgvr.so``.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); the C++ host sources go
through nvcc's host compiler. Translation units compile in parallel and are
linked with the static CUDA runtime, so the library needs nothing but the
driver at run time.
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
OUT = PKG / "_lib"
LIB = OUT / "libgvr.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libgvr")
    return cand


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    cmd = [_nvcc(), *ARCH, *COMMON, *extra, "-DGVR_BUILDING", "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip() and os.environ.get("GVR_BUILD_VERBOSE"):
        sys.stderr.write(res.stderr)


def build(force: bool = False, extra: list[str] | None = None) -> Path:
    """Compile csrc/ into libgvr.so; skip when the library is newer than every source."""
    extra = list(extra or [])
    srcs = sources()
    deps = srcs + sorted(CSRC.glob("*.h")) + [PKG.parent / "include" / "gvr.h", Path(__file__)]
    if not force and LIB.exists():
        newest = max(p.stat().st_mtime for p in deps)
        if LIB.stat().st_mtime > newest:
            return LIB
    objdir = OUT / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    objs = [objdir / (s.stem + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], extra), zip(srcs, objs)))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
