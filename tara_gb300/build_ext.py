"""Build libtara.so (CUDA, sm_103a) in-tree, and the CPU oracle used by the tests.

Translation units compile in parallel into ``tara_gb300/_build`` and link into
``tara_gb300/libtara.so``.  The library exposes only the C ABI of
``include/tara.h``; it has no Python or torch dependency.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libtara.so"
ORACLE = ROOT / "oracle"
# The reference checkout (for the FFTW-backed oracle only): named by the
# TARA_REFERENCE environment variable; without it oracle/_ref is not built.
REFERENCE = Path(os.environ["TARA_REFERENCE"]) if os.environ.get("TARA_REFERENCE") else None

SOURCES = ["launch_fp64.cu", "launch_fp64_r8.cu", "launch_fp32.cu", "launch_fp32_r8.cu", "launch_df64.cu", "solver2d.cu", "generic2d.cu", "capi.cu", "noalloc.cu", "mhd3d.cu",
           "ensemble.cu", "ens_persistent.cu", "fno.cu", "fno_tc.cu", "fno_fused.cu", "fno_dft_tc.cu", "fno_head_tc.cu", "closure.cu", "particles.cu", "coh2d.cu", "com2d.cu", "ini.cpp",
           "driver.cpp"]
EXE = PKG / "tara"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    # host code keeps IEEE double without FMA contraction (wavenumber tables
    # must equal the oracle's on x86 and Arm alike)
    "-Xcompiler", "-fPIC,-ffp-contract=off,-Wall,-Wextra",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stamp(paths) -> str:
    h = hashlib.sha1()
    for p in sorted(paths):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(NVCC_FLAGS).encode())
    return h.hexdigest()


def _compile(src: Path, obj: Path) -> str:
    """Compile one translation unit; returns the compiler's warnings (if any)."""
    cmd = [nvcc(), *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return "\n".join(l for l in (r.stdout + r.stderr).splitlines() if "warning" in l.lower())


def build_lib(force: bool = False, verbose: bool = False) -> Path:
    deps = (list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) +
            list(CSRC.glob("*.cpp")))
    deps.append(ROOT / "include" / "tara.h")
    stamp = _stamp(deps)
    stamp_file = BUILD / "stamp"
    if not force and LIB.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return LIB
    BUILD.mkdir(exist_ok=True)
    objs = [BUILD / (s.rsplit(".", 1)[0] + ".o") for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(_compile, CSRC / s, o) for s, o in zip(SOURCES, objs)]
        for f in futs:
            warn = f.result()
            if warn:
                print(warn, file=sys.stderr)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # the `tara` executable (input.ini driver) links the library by relative rpath
    cmd = [nvcc(), *ARCH, "-o", str(EXE), str(CSRC / "tara_main.cpp"), f"-L{PKG}", "-ltara",
           "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"tara executable link failed:\n{r.stdout}\n{r.stderr}")
    stamp_file.write_text(stamp)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(verbose: bool = False) -> None:
    """Oracle (test infrastructure): the own-FFT restatement everywhere, and the
    FFTW-from-reference-sources build only where TARA_REFERENCE names a
    reference tree that exists."""
    r = subprocess.run(["make", "-s", "-C", str(ORACLE), "port"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if REFERENCE is not None and (REFERENCE / "lib" / "fftw" / "api" / "fftw3.h").exists():
        jobs = str(os.cpu_count() or 4)
        r = subprocess.run(["make", "-s", "-j", jobs, "-C", str(ORACLE), "ref", f"REF={REFERENCE}"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle/_ref build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built oracle")


def build(force: bool = False, verbose: bool = False) -> None:
    build_lib(force=force, verbose=verbose)
    build_oracle(verbose=verbose)


if __name__ == "__main__":
    build(force=True, verbose=True)
