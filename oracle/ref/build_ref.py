"""Build and run the reference programs as oracle binaries (TEST INFRASTRUCTURE).

The reference keeps its parameters as compile-time `const` globals
(mpi_evolution.cpp:15-60, evolution.cpp:23-58, mooreEvol.cpp:19-42,
moore_mpi_evolution.cpp:15-65) and writes its output next to its own source
file (dir_path from __FILE__, evolution.cpp:72-73).  So each configuration is
built from a copy of the reference source, made in a scratch directory outside
the repository, with the chosen `const` values substituted; nothing else in
the source changes.  Two headers of this repository are added on the compile
line:

  * oracle/ref/axr_hooks.h (force-included): ofstream at 17 digits;
  * oracle/ref/mpi_stub/mpi.h: single-rank MPI whose MPI_Finalize() dumps the
    fields (the MPI programs never write them).

Binaries go to oracle/_ref/ (git-ignored).  The reference directory is only
read; it exists in this development container, not on the GPU machines, which
use the committed fixtures in tests/golden/ instead.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
REF_OUT = ORACLE / "_ref"
# The reference checkout: given by the caller (set_reference) or the
# AXIONS_REFERENCE environment variable; there is no default location.
REFERENCE: Path | None = Path(os.environ["AXIONS_REFERENCE"]) if os.environ.get("AXIONS_REFERENCE") else None
SCRATCH = Path(os.environ.get("AXIONS_REF_SCRATCH", "/tmp/axions_ref"))


def set_reference(path) -> None:
    """Use the reference checkout at `path` for the builds below."""
    global REFERENCE
    REFERENCE = Path(path)

# program -> (extra sources that lie in the reference dir, MPI field list)
PROGRAMS = {
    "mpi_evolution": ([], "totSize,haloSize,coreSize,phi,theta"),
    "moore_mpi_evolution": ([], "totSize,haloSize,coreSize,phi1,phi2,theta"),
    "evolution": (["array.cpp"], None),
    "mooreEvol": (["array.cpp"], None),
    # ic_w_evolution.cpp:79 builds its IC in-process with ic_func() (ic_func.cpp:18)
    "ic_w_evolution": (["ic_func.cpp", "array.cpp"], None),
    "initialConditions": (["array.cpp"], None),
    "singleSemiAnalytic": (["array.cpp"], None),
}


def reference_available() -> bool:
    return REFERENCE is not None and (REFERENCE / "mpi_evolution.cpp").is_file()


def _require_reference() -> Path:
    if not reference_available():
        raise RuntimeError("reference sources not found: pass the reference directory (set_reference, "
                           "--reference) or set AXIONS_REFERENCE")
    return REFERENCE


def _fmt(v) -> str:
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, str):
        return '"' + v + '"'
    if isinstance(v, float):
        return repr(v)
    if isinstance(v, (list, tuple)):
        return "{" + ", ".join(_fmt(float(x)) for x in v) + "}"
    return str(v)


def substitute_consts(src: str, consts: dict) -> str:
    """Replace the initialiser of `[const] <type> NAME = ...;` lines (the
    boundary-condition strings of ic_w_evolution.cpp:44-45 are not const)."""
    out = src
    for name, val in consts.items():
        pat = re.compile(r"^(\s*(?:const\s+)?(?:int|double|bool|string)\s+" + re.escape(name)
                         + r"(?:\[\d*\])?\s*=\s*)([^;]*)(;)", re.MULTILINE)
        out, n = pat.subn(lambda m: m.group(1) + _fmt(val) + m.group(3), out, count=1)
        if n != 1:
            raise KeyError(f"const {name} not found")
    return out


def build(program: str, tag: str, consts: dict, extra_consts: dict | None = None) -> Path:
    """Build `program` with `consts`; return the binary path.  `extra_consts`
    maps an extra source (e.g. "ic_func.cpp") to the constants substituted in
    a copy of it."""
    if program not in PROGRAMS:
        raise ValueError(program)
    extra, fields = PROGRAMS[program]
    _require_reference()
    work = SCRATCH / tag
    if work.exists():
        shutil.rmtree(work)
    (work / "Data").mkdir(parents=True)
    (work / "GifData").mkdir()
    src = (REFERENCE / f"{program}.cpp").read_text()
    (work / f"{program}.cpp").write_text(substitute_consts(src, consts))
    REF_OUT.mkdir(exist_ok=True)
    binary = REF_OUT / tag
    cmd = ["g++", "-O3", "-fopenmp", "-std=c++17", "-w",
           "-include", str(HERE / "axr_hooks.h"),
           "-I", str(REFERENCE)]
    if fields:
        cmd += ["-I", str(HERE / "mpi_stub"), f"-DAXR_FIELDS={fields}"]
    sources = [str(work / f"{program}.cpp")]
    for e in extra:
        if extra_consts and e in extra_consts:
            (work / e).write_text(substitute_consts((REFERENCE / e).read_text(), extra_consts[e]))
            sources.append(str(work / e))
        else:
            sources.append(str(REFERENCE / e))
    cmd += sources
    cmd += ["-o", str(binary)]
    subprocess.run(cmd, check=True)
    return binary


def run(tag: str, stdin: str = "", ic_lines: list[str] | None = None, ic_name: str = "ic.txt",
        threads: int = 1, timeout: int = 600) -> Path:
    """Run a built binary in its scratch dir; return the scratch dir."""
    work = SCRATCH / tag
    if ic_lines is not None:
        (work / "Data" / ic_name).write_text("\n".join(ic_lines) + "\n")
    env = dict(os.environ)
    env["OMP_NUM_THREADS"] = str(threads)
    env["AXR_DUMP"] = str(work / "Data" / "axr_fields.bin")
    subprocess.run([str(REF_OUT / tag)], input=stdin.encode(), cwd=work, env=env, check=True,
                   stdout=subprocess.DEVNULL, timeout=timeout)
    return work


def read_columns(path: Path):
    import numpy as np
    txt = path.read_text().split()
    return np.array([float(t) for t in txt], dtype=np.float64)


def build_defaults() -> list[Path]:
    """Build each reference program once with a small configuration (the build
    check of __graft_entry__.build(); tests/golden/make_golden.py builds and runs
    the configurations of the fixtures)."""
    small = {"nx": 8, "ny": 8, "nz": 8, "nt": 2}
    out = [build("mpi_evolution", "mpi_evolution_small", small),
           build("moore_mpi_evolution", "moore_mpi_evolution_small", small),
           build("evolution", "evolution_small", small),
           build("mooreEvol", "mooreEvol_small", small),
           build("ic_w_evolution", "ic_w_evolution_small", dict(small, makeGif=False),
                 {"ic_func.cpp": {"ic_type": "random"}})]
    return out
