"""Builds libfbp.so (and the C++ host shim) in-tree with nvcc for sm_103a.

Each CUDA translation unit compiles in parallel to an object under
``fasterbackprojection_gb300/_build/``; the objects link into
``fasterbackprojection_gb300/_lib/libfbp.so``.  Rebuilds only what changed
(sources newer than their object, or a header newer than anything).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
CPP = PKG / "cpp"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIBFBP = LIBDIR / "libfbp.so"
LIBFBP_HOST = LIBDIR / "libfbp_host.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "--expt-relaxed-constexpr",
                     "-diag-suppress", "177"]


def _nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(home) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found: set CUDA_HOME")
    return found


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile every .cu under csrc/ and link libfbp.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    srcs = sorted(CSRC.glob("*.cu"))
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if _stale(o, [s] + headers)]

    def compile_one(so):
        s, o = so
        cmd = [nvcc, *NVCC_FLAGS, "-I", str(ROOT / "include"), "-c", str(s), "-o", str(o)]
        if verbose:
            print(" ".join(cmd), flush=True)
        _run(cmd)

    jobs = jobs or max(1, min(len(todo), os.cpu_count() or 4))
    if todo:
        with ThreadPoolExecutor(max_workers=jobs) as ex:
            list(ex.map(compile_one, todo))
    if todo or _stale(LIBFBP, objs):
        tmp = LIBFBP.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs)])
        os.replace(tmp, LIBFBP)
    _build_host_shim(verbose)
    return LIBFBP


def _build_host_shim(verbose: bool) -> None:
    """The C++ classes mirroring the reference's host interface (cpp/)."""
    srcs = sorted(CPP.glob("*.cpp"))
    if not srcs:
        return
    deps = srcs + sorted(CPP.glob("*.hpp")) + [LIBFBP, ROOT / "include" / "fbp.h"]
    if not _stale(LIBFBP_HOST, deps):
        return
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", str(ROOT / "include"), "-I", str(CPP),
           "-I", f"{home}/include", *map(str, srcs), "-o", str(LIBFBP_HOST), "-L", str(LIBDIR), "-lfbp",
           f"-Wl,-rpath,$ORIGIN", "-L", f"{home}/lib64", "-lcudart", f"-Wl,-rpath,{home}/lib64"]
    if verbose:
        print(" ".join(cmd), flush=True)
    _run(cmd)


def build_oracle(verbose: bool = False) -> None:
    """CPU oracle + reference-kernel harness (test infrastructure)."""
    oracle = ROOT / "oracle"
    _run(["make", "-s", "-C", str(oracle), "all"])
    # The reference checkout beside this repository (../reference), unless
    # FBP_REFERENCE_DIR names its FasterBackprojection/ directory.
    ref_dir = Path(os.environ.get("FBP_REFERENCE_DIR", str(ROOT.parent / "reference" / "FasterBackprojection")))
    if ref_dir.is_dir():
        _run(["make", "-s", "-C", str(oracle), "ref", f"REF_DIR={ref_dir}"])


if __name__ == "__main__":
    build(verbose=True)
    build_oracle(verbose=True)
    print(LIBFBP)
