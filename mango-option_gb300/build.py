"""Build the in-tree engine library (and, for tests, the CPU oracle).

libmango_gpu.so: every .cu in csrc/ through nvcc for sm_103a only, the host
grid code through g++ with -ffp-contract=off (grids must match the reference
bit for bit), linked with the static CUDA runtime.  Translation units compile
in parallel; the whole build takes well under a minute.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libmango_gpu.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "libmango_oracle.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(target: pathlib.Path, sources: list[pathlib.Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_engine(force: bool = False, verbose: bool = False) -> pathlib.Path:
    OUT.mkdir(parents=True, exist_ok=True)
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    headers = sorted(CSRC.glob("*.hpp")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "mango_gpu.h"]
    if not force and not _stale(LIB, cu + cpp + headers + [pathlib.Path(__file__)]):
        return LIB
    nvcc = _nvcc()
    inc = ["-I", str(CSRC), "-I", str(ROOT / "include")]
    jobs = []
    for src in cu:
        obj = OUT / (src.stem + ".o")
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", *inc,
                     "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = OUT / (src.stem + ".o")
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", *inc,
                     "-I", "/usr/local/cuda/include", "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    objs = [str(OUT / (s.stem + ".o")) for s in cu + cpp]
    tmp = OUT / "libmango_gpu.so.tmp"
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *objs, "-lpthread"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(force: bool = False) -> pathlib.Path:
    """Compile the C restatement used by tests as the checker (never by the
    engine)."""
    src = ORACLE_DIR / "mango_oracle.c"
    hdr = ORACLE_DIR / "mango_oracle.h"
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    if force or _stale(ORACLE_LIB, [src, hdr]):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-o", str(tmp), str(src), "-lm"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def reference_dir() -> pathlib.Path | None:
    """The reference tree: $MANGO_REFERENCE_DIR, else a checkout named
    `reference` beside this repository; None when neither exists (the GPU
    host never has it)."""
    env = os.environ.get("MANGO_REFERENCE_DIR")
    for cand in ([pathlib.Path(env)] if env else []) + [ROOT.parent / "reference"]:
        if (cand / "src" / "option" / "american_option.cpp").exists():
            return cand
    return None


def build_reference_oracle() -> pathlib.Path | None:
    """Compile the reference's own sources into oracle/_ref when the
    reference tree is present."""
    ref = reference_dir()
    if ref is None:
        return None
    _run(["make", "-s", "-C", str(ORACLE_DIR / "ref"), f"REF={ref}", "-j8"])
    build_reference_parquet(ref)
    return ORACLE_DIR / "_ref" / "libmango_ref.so"


def build_reference_parquet(ref: pathlib.Path) -> pathlib.Path | None:
    """The reference's Parquet writer and reader, against the Arrow C++
    libraries pyarrow bundles, when pyarrow is importable (its version's
    library names must match the ones found)."""
    try:
        import pyarrow as pa
    except ImportError:
        return None
    lib_dir = pa.get_library_dirs()[0]
    sover = [p.name.split(".so.")[1] for p in pathlib.Path(lib_dir).glob("libparquet.so.*")
             if p.name.split(".so.")[1].isdigit()]
    if not sover:
        return None
    _run(["make", "-s", "-C", str(ORACLE_DIR / "ref"), f"REF={ref}", "parquet",
          f"ARROW_INC={pa.get_include()}", f"ARROW_LIB={lib_dir}", f"ARROW_SOVER={sover[0]}"])
    return ORACLE_DIR / "_ref" / "libmango_ref_parquet.so"


if __name__ == "__main__":
    build_engine(force=True, verbose=True)
    build_oracle(force=True)
