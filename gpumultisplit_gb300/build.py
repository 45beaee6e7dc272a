"""Builds libgpumultisplit.so (sm_103a) in-tree with nvcc.

Every ``csrc/*.cu`` translation unit is compiled in parallel, then linked into
``gpumultisplit_gb300/lib/libgpumultisplit.so``.  A rebuild happens only when a
source or header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
INCLUDE = PKG_DIR.parent / "include"
LIB_DIR = PKG_DIR / "lib"
LIB_PATH = LIB_DIR / "libgpumultisplit.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE)]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc", "/usr/local/cuda-13.0/bin/nvcc"):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gpumultisplit_gb300")


# inst_batch.cu is compiled once per (identifier kind, tile variant),
# inst_wide.cu and inst_big.cu once per identifier kind; the counts match NUM_KINDS in
# gms_device.cuh and kNumTileVariants in ms_host.h.
BATCH_INST = "inst_batch.cu"
WIDE_INST = "inst_wide.cu"
BIG_INST = "inst_big.cu"
NUM_KINDS = 6
NUM_TILE_VARIANTS = 4


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _units() -> list[tuple[Path, str, list[str]]]:
    """(source, object stem, extra flags) of every translation unit."""
    units = []
    for s in _sources():
        if s.name == BATCH_INST:
            for k in range(NUM_KINDS):
                for v in range(NUM_TILE_VARIANTS):
                    units.append((s, f"{s.stem}_k{k}_v{v}", [f"-DGMS_INST_KIND={k}", f"-DGMS_INST_VARIANT={v}"]))
        elif s.name in (WIDE_INST, BIG_INST):
            for k in range(NUM_KINDS):
                units.append((s, f"{s.stem}_k{k}", [f"-DGMS_INST_KIND={k}"]))
        else:
            units.append((s, s.stem, []))
    return units


def _deps() -> list[Path]:
    return _sources() + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def needs_build() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _deps())


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")
    if verbose and r.stdout.strip():
        print(r.stdout, flush=True)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile the CUDA library if needed and return its path."""
    if not force and not needs_build():
        return LIB_PATH
    nvcc = nvcc_path()
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    stale = LIB_DIR / "obj"  # objects of earlier builds, which kept them next to the library
    if stale.is_dir():
        shutil.rmtree(stale)
    with tempfile.TemporaryDirectory(prefix="gms_build_") as tmp_dir:
        _compile_and_link(nvcc, Path(tmp_dir), verbose, extra_flags)
    return LIB_PATH


def _compile_and_link(nvcc: str, obj_dir: Path, verbose: bool, extra_flags: list[str] | None) -> None:
    flags = ARCH_FLAGS + NVCC_FLAGS + list(extra_flags or [])
    units = _units()
    # Largest units first so the parallel build ends sooner.
    units.sort(key=lambda u: (not u[1].startswith("inst_"), u[1].startswith(BATCH_INST[:-3])))
    objs = [obj_dir / (stem + ".o") for _, stem, _ in units]
    jobs = max(1, min(len(units), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_run, [nvcc, *flags, *extra, "-c", str(s), "-o", str(o)], verbose)
                for (s, _, extra), o in zip(units, objs)]
        for f in futs:
            f.result()
    tmp = LIB_DIR / (LIB_PATH.name + ".tmp")
    _run([nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs)], verbose)
    os.replace(tmp, LIB_PATH)


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
