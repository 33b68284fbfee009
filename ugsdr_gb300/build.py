"""Build recipe for libugsdr_cuda.so (sm_103a) and the CPU oracle.

nvcc compiles each translation unit of ugsdr_gb300/csrc in parallel and
links them into ugsdr_gb300/_lib/libugsdr_cuda.so (in-tree; git-ignored).
Objects are rebuilt only when a source or header changed.
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
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "libugsdr_cuda.so"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "--expt-relaxed-constexpr", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I", str(ROOT / "include")]
SOURCES = ["acq.cu", "ops.cu", "ctx.cu", "track.cu", "serve.cpp", "codes.cpp", "noalloc.cu", "refine.cpp", "jamming.cu", "observables.cu", "tc_dft.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _headers_digest() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + list((ROOT / "include").glob("*.h"))):
        h.update(p.read_bytes())
    h.update(" ".join(NVCC_FLAGS + ARCH).encode())
    return h.hexdigest()[:16]


def _compile(src: Path, obj: Path, stamp: Path, digest: str, verbose: bool) -> None:
    key = digest + hashlib.sha256(src.read_bytes()).hexdigest()[:16]
    if obj.exists() and stamp.exists() and stamp.read_text() == key:
        return
    cmd = [nvcc(), *NVCC_FLAGS, *ARCH, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    stamp.write_text(key)


GALILEO_TABLE = PKG / "data" / "galileo_e1_memory_codes.bin"


def _table_source(obj_dir: Path) -> Path:
    """The Galileo E1B/E1C memory-code table as a C++ array (generated)."""
    src = obj_dir / "galileo_table.cpp"
    data = GALILEO_TABLE.read_bytes()
    body = ",".join(str(b) for b in data)
    text = ("// generated by ugsdr_gb300/build.py from data/galileo_e1_memory_codes.bin\n"
            f"extern const unsigned char ugsdr_galileo_e1_table[{len(data)}] = {{{body}}};\n")
    if not src.exists() or src.read_text() != text:
        src.write_text(text)
    return src


def build_library(verbose: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    obj_dir = OUT_DIR / "obj"
    obj_dir.mkdir(exist_ok=True)
    digest = _headers_digest()
    sources = [CSRC / s for s in SOURCES if (CSRC / s).exists()] + [_table_source(obj_dir)]
    objs = [obj_dir / (s.name + ".o") for s in sources]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, s, o, o.with_suffix(".stamp"), digest, verbose) for s, o in zip(sources, objs)]
        for f in futs:
            f.result()
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB) + ".tmp", *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(str(LIB) + ".tmp", LIB)
    return LIB


def reference_dir() -> Path:
    """The reference checkout: $UGSDR_REF_DIR, else a sibling directory
    named `reference` beside this repository."""
    env = os.environ.get("UGSDR_REF_DIR")
    return Path(env) if env else ROOT.parent / "reference"


def build_oracle(verbose: bool = False) -> None:
    """CPU oracle (test infrastructure): the port always, the reference build
    only where the reference sources exist."""
    r = subprocess.run(["make", "-s", "-C", str(ORACLE), "all"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    ref_dir = reference_dir()
    if (ref_dir / "src" / "acquisition" / "fse.hpp").exists():
        r = subprocess.run(["make", "-s", "-C", str(ORACLE), "ref", f"REF_DIR={ref_dir}"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")


def build_all(verbose: bool = False) -> None:
    build_library(verbose)
    build_oracle(verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print(LIB)
