"""Build recipes for the native parts of the repository.

- ``libpdgb.so``: the engine (CUDA kernels for sm_103a + C ABI), compiled with
  nvcc, one translation unit per process in parallel, then linked.
- ``oracle/liboracle.so``: the CPU oracle (test infrastructure), g++.
- ``oracle/_ref/libref_pd.so``: the reference's own PD kernels compiled as
  C++ (only where the reference sources are present; test infrastructure).
- ``baseline/_build/librefgpu.so``: the reference's GPU PD step restated with
  cuSOLVER's sparse Cholesky, timed beside the engine (a baseline, not part
  of the engine).

Nothing here downloads anything; the only tools used are nvcc and g++.
"""
from __future__ import annotations

import concurrent.futures as _cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent.parent
CSRC = PKG_DIR.parent / "csrc"
LIB_DIR = PKG_DIR / "_lib"
LIB_PATH = LIB_DIR / "libpdgb.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"
BASELINE_DIR = ROOT / "baseline"
REFGPU_LIB = BASELINE_DIR / "_build" / "librefgpu.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str], cwd: Path | None = None) -> None:
    proc = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def engine_sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def build_engine(force: bool = False, verbose: bool = False) -> Path:
    srcs = engine_sources()
    deps = srcs + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "pdgb.h", Path(__file__)]
    if not force and not _stale(LIB_PATH, deps):
        return LIB_PATH
    nvcc = _nvcc()
    obj_dir = LIB_DIR / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    common = ARCH_FLAGS + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off,-fopenmp",
                           "-I", str(ROOT / "include")]

    # the collision narrow phase matches the CPU oracle operation for operation
    per_file = {"ccd.cu": ["--fmad=false"]}

    def compile_one(src: Path) -> Path:
        obj = obj_dir / (src.name + ".o")
        cmd = [nvcc] + common + per_file.get(src.name, []) + ["-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        _run(cmd)
        return obj

    with _cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    _run([nvcc] + ARCH_FLAGS + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lcudart", "-lgomp"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_oracle(force: bool = False) -> Path:
    srcs = [ORACLE_DIR / "pd_oracle.cpp", ORACLE_DIR / "ccd_oracle.cpp"]
    deps = srcs + [ORACLE_DIR / "pd_oracle.h"]
    if not force and not _stale(ORACLE_LIB, deps):
        return ORACLE_LIB
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    _run(["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"] + [str(x) for x in srcs]
         + ["-o", str(tmp)])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference_harness(force: bool = False) -> Path | None:
    """Builds oracle/_ref from the reference's sources when they are present
    (the recipe oracle/build_ref.sh finds them: its argument,
    $PDGB_REFERENCE_ROOT, or where this project's build container mounts
    them; elsewhere it builds nothing)."""
    script = ORACLE_DIR / "build_ref.sh"
    if not script.exists():
        return None
    out = ORACLE_DIR / "_ref" / "libref_pd.so"
    deps = [script, ORACLE_DIR / "pd_oracle.cpp"] + sorted((ORACLE_DIR / "refshim").glob("*.*"))
    if not force and not _stale(out, [d for d in deps if d.exists()]):
        return out
    args = ["bash", str(script)]
    if os.environ.get("PDGB_REFERENCE_ROOT"):
        args.append(os.environ["PDGB_REFERENCE_ROOT"])
    _run(args, cwd=ORACLE_DIR)
    return out if out.exists() else None


def reference_root() -> Path | None:
    """Root of the reference's sources this checkout's oracle/_ref was built
    from ($PDGB_REFERENCE_ROOT first), or None where they are absent."""
    env = os.environ.get("PDGB_REFERENCE_ROOT")
    if env and Path(env).is_dir():
        return Path(env)
    rec = ORACLE_DIR / "_ref" / "REFERENCE_ROOT"
    if rec.exists():
        p = Path(rec.read_text().strip())
        if p.is_dir():
            return p
    return None


def build_refgpu(force: bool = False) -> Path:
    src = BASELINE_DIR / "refgpu.cu"
    deps = [src, CSRC / "rotation.cuh", Path(__file__)]
    if not force and not _stale(REFGPU_LIB, deps):
        return REFGPU_LIB
    REFGPU_LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = REFGPU_LIB.with_suffix(".so.tmp")
    _run([_nvcc()] + ARCH_FLAGS + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                   "-Wno-deprecated-declarations", "-I", str(CSRC), "-shared", str(src), "-o",
                                   str(tmp), "-lcusolver", "-lcusparse"])
    os.replace(tmp, REFGPU_LIB)
    return REFGPU_LIB


def build_all(force: bool = False) -> None:
    with _cf.ThreadPoolExecutor(max_workers=4) as ex:
        futs = [ex.submit(build_engine, force), ex.submit(build_oracle, force),
                ex.submit(build_reference_harness, force), ex.submit(build_refgpu, force)]
        for f in futs:
            f.result()
