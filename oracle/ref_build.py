"""Recipe for the reference's own GPU build of the hot path (test infrastructure only).

The reference computes the hologram path with cuFFT, cuBLAS (Cgemm3m), cuSOLVER (Cheevd) and
thrust, called from a handful of translation units under ``Backend/cuda_sources`` and
``Backend/sources``. This recipe compiles those files unmodified, with the shim headers in
``oracle/ref_shims`` standing in for the logging / JSON / Windows headers they include, together
with ``oracle/ref_pipe.cu`` (the cycle driver, this repository's code) into
``oracle/_ref/libhvref.so``. Tests and the bench compare the product with it on the same inputs.

Two steps, because the reference tree exists only in the build container and the GPU machine is an
Arm machine (host objects built here do not run there):

* ``stage()`` (needs the reference tree): copies the listed translation units and the headers they
  include, unmodified, into the git-ignored ``oracle/_ref/src`` (the tree layout is kept). Nothing
  from there is committed; the folder travels to the GPU machine with the working copy.
* ``build()`` compiles ``oracle/_ref/src`` + ``ref_pipe.cu`` with nvcc for sm_103a and links against
  cuFFT / cuBLAS / cuSOLVER.

    python oracle/ref_build.py [--reference DIR] [--stage-only]
"""

from __future__ import annotations

import hashlib
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
SHIMS = HERE / "ref_shims"
OUT = HERE / "_ref"
SRC = OUT / "src"
LIB = OUT / "libhvref.so"
DRIVER = HERE / "ref_pipe.cu"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# the reference's hot-path translation units (paths inside the reference tree)
UNITS = [f"Backend/cuda_sources/{n}.cu" for n in (
    "masks", "fresnel_transform", "angular_spectrum", "apply_mask", "tools_conversion", "tools_compute",
    "shift_corners", "stft", "percentile", "contrast_correction", "map", "tools_unwrap", "complex_utils", "tools")] + [
    "Backend/sources/compute/matrix_operations.cc",
    "Backend/sources/compute/compute_bundles_2d.cc",
    "Backend/sources/tools/hardware_limits.cc",
    "Backend/sources/tools/cuda_tools/cublas_handle.cc",
    "Backend/sources/tools/cuda_tools/cusolver_handle.cc",
    "Backend/sources/tools/cuda_tools/cufft_handle.cc",
]
INCLUDE_ROOTS = ["Backend/includes", "Backend/cuda_includes", "Camera/include"]


def default_reference() -> Path:
    return Path(os.environ.get("HV_REFERENCE_TREE", "/root/reference"))


def _include_dirs(tree: Path) -> list[Path]:
    dirs = []
    for r in INCLUDE_ROOTS:
        for d, _, _ in os.walk(tree / r):
            dirs.append(Path(d))
    return dirs


def stage(reference: Path | None = None) -> bool:
    """Copies the translation units and their quoted includes (transitively, shims excluded) from
    the reference tree into oracle/_ref/src. Returns False when the reference tree is absent."""
    tree = reference or default_reference()
    if not (tree / UNITS[0]).is_file():
        return False
    shimmed = {p.name for p in SHIMS.glob("*.hh")}
    dirs = _include_dirs(tree)
    seen: set[Path] = set()
    todo = [tree / u for u in UNITS]
    # the headers the cycle driver includes come from the reference tree as well
    driver_incs = re.findall(r'#\s*include\s+"([^"]+)"', DRIVER.read_text())
    for inc in driver_incs:
        hit = next((d / inc for d in dirs if (d / inc).is_file()), None)
        if hit is not None and Path(inc).name not in shimmed:
            todo.append(hit.resolve())
    while todo:
        f = todo.pop()
        if f in seen:
            continue
        seen.add(f)
        text = f.read_text(errors="replace")
        for m in re.finditer(r'#\s*include\s+"([^"]+)"', text):
            inc = m.group(1).replace("\\", "/")
            if Path(inc).name in shimmed:
                continue
            for cand in [f.parent / inc] + [d / inc for d in dirs]:
                if cand.is_file():
                    todo.append(cand.resolve())
                    break
    if SRC.exists():
        shutil.rmtree(SRC)
    for f in seen:
        if f == DRIVER:
            continue
        dst = SRC / f.relative_to(tree.resolve())
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(f, dst)
    (SRC / "STAGED_FROM").write_text(f"{tree}\n")
    return True


def staged() -> bool:
    return (SRC / UNITS[0]).is_file()


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _flags() -> list[str]:
    inc = [f"-I{SHIMS}"]
    for r in INCLUDE_ROOTS:
        for d, _, _ in os.walk(SRC / r):
            inc.append(f"-I{d}")
    return ["-O3", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC", "-include", "cfloat",
            "-include", "cmath", "-DNDEBUG", *inc]


def _digest() -> str:
    h = hashlib.sha256()
    for p in sorted(list(SRC.rglob("*")) + list(SHIMS.glob("*")) + [DRIVER, Path(__file__)]):
        if p.is_file():
            h.update(str(p.relative_to(HERE)).encode())
            h.update(p.read_bytes())
    h.update(" ".join(ARCH + _flags()).encode())
    return h.hexdigest()


def build(force: bool = False) -> Path:
    """Compiles the staged reference units and the cycle driver into oracle/_ref/libhvref.so."""
    if not staged():
        raise RuntimeError("the reference sources are not staged in oracle/_ref/src (run stage() where the "
                           "reference tree exists)")
    stamp = OUT / "build.sha256"
    digest = _digest()
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == digest:
        return LIB
    objdir = OUT / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    flags = _flags()

    def compile_one(src: Path) -> Path:
        obj = objdir / (src.name + ".o")
        cmd = [cc, *ARCH, *flags, "-x", "cu", "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr[-4000:]}")
        return obj

    srcs = [SRC / u for u in UNITS] + [DRIVER]
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcufft", "-lcublas", "-lcusolver"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    stamp.write_text(digest)
    return LIB


if __name__ == "__main__":
    ref = None
    if "--reference" in sys.argv:
        ref = Path(sys.argv[sys.argv.index("--reference") + 1])
    if stage(ref):
        print("staged", SRC)
    if "--stage-only" not in sys.argv:
        print(build(force="--force" in sys.argv))
