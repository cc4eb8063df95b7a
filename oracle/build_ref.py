"""ORACLE -- test infrastructure.  Recipe that compiles the reference program
itself (jijn/phasefield_coarsening phasefield.c) as a second, independent
oracle and as the CPU baseline.

The reference fixes its configuration at compile time with unguarded
#defines and const locals, and it needs MPI and libhdf5, neither of which is
installed.  So the recipe reads phasefield.c where it lies, applies a fixed
list of one-line substitutions, writes the patched translation unit to
oracle/_ref/ (git-ignored; nothing from the reference is committed) and
compiles it with gcc against the <hdf5.h> stand-in in oracle/hdf5_shim/
(over the oracle's own HDF5 code, h5ref.c: no product code is linked).
The reference source is read from $PPF_REFERENCE_SRC when that is set.

Substitutions (each must match exactly once, else the build fails):
  phasefield.c:13      USE_MPI 1 -> 0 (serial build: MPI is absent)
  phasefield.c:15      USE_BC_TYPE -> the requested BC
  phasefield.c:48-50   NX/NY/NZ of the serial build -> the requested grid
  phasefield.c:92      dt -> the requested expression (default unchanged)
  phasefield.c:104     n_iter, n_save -> requested
  phasefield.c:105     n_iter_init -> requested (default unchanged)
  phasefield.c:1032    H5Dread(dataset_id_S, ... etaL) -> dataset_id_L, unless
                       the unfixed read is requested (the reference's bug:
                       /etaL is read through the closed /etaS identifier, so
                       etaL keeps its initial value 1.0)
  + #include <math.h>/<time.h> and a CLOCK_MONOTONIC timer around the main
    loop (:178-258), printed as "ppf-ref loop seconds: S" on stderr
  + optionally "#pragma omp parallel for" on the three passes of
    sweep_fields (:325, :347, :393); each pass writes every cell from values
    that pass does not write, so the arithmetic is unchanged.
The arithmetic of sweep_fields / sweep_fields_c (:301-476) is untouched.

On a machine without the reference sources (the GPU host), a patched unit
that was generated earlier in oracle/_ref/ is compiled as is.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
# where the reference source lies; PPF_REFERENCE_SRC overrides it
REF_SRC = os.environ.get("PPF_REFERENCE_SRC", "/root/reference/phasefield.c")
OUT_DIR = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "hdf5_shim")
H5REF = os.path.join(SHIM, "h5ref.c")


def _sub_once(src: str, old: str, new: str) -> str:
    n = src.count(old)
    if n != 1:
        raise RuntimeError(f"reference patch anchor found {n} times: {old!r}")
    return src.replace(old, new)


def _omp_pragmas(src: str) -> str:
    start = src.index("int sweep_fields(double")
    end = src.index("int sweep_fields_c(double")
    body = src[start:end]
    lines = body.split("\n")
    out = []
    seen_a = 0
    for ln in lines:
        if ln == "    for (i=0;i<NI+2;i++){":
            out.append("#pragma omp parallel for private(j,k)")
            seen_a += 1
        elif ln == "    for (i=1;i<=NI;i++){":
            out.append("#pragma omp parallel for private(j,k,tmp4,cS,cL,fS,fL,dmu)")
        out.append(ln)
    if seen_a != 2:
        raise RuntimeError("sweep_fields loop anchors not found")
    return src[:start] + "\n".join(out) + src[end:]


def patch(src: str, nz: int, ny: int, nx: int, bc: int, n_iter: int, n_save: int,
          n_iter_init: int | None, dt_expr: str | None, fix_etaL: bool, omp: bool) -> str:
    s = _sub_once(src, "#define USE_MPI 1", "#define USE_MPI 0")
    s = _sub_once(s, "#define USE_BC_TYPE 1 ", f"#define USE_BC_TYPE {int(bc)} ")
    s = _sub_once(s, "#define NX 100", f"#define NX {int(nx)}")
    s = _sub_once(s, "#define NY 100", f"#define NY {int(ny)}")
    s = _sub_once(s, "#define NZ 100", f"#define NZ {int(nz)}")
    if dt_expr is not None:
        s = _sub_once(s, "const double dt = 0.125*dx*dx/DL;", f"const double dt = {dt_expr};")
    s = _sub_once(s, "const long n_iter=5000001L,n_save=50000L;",
                  f"const long n_iter={int(n_iter)}L,n_save={int(n_save)}L;")
    if n_iter_init is not None:
        s = _sub_once(s, "const long n_iter_init = 100000000L;",
                      f"const long n_iter_init = {int(n_iter_init)}L;")
    if fix_etaL:
        s = _sub_once(s, "H5Dread(dataset_id_S,H5T_IEEE_F64LE,memspace_id,filespace_id,H5P_DEFAULT,etaL);",
                      "H5Dread(dataset_id_L,H5T_IEEE_F64LE,memspace_id,filespace_id,H5P_DEFAULT,etaL);")
    s = _sub_once(s, "#include <string.h>\n", "#include <string.h>\n#include <math.h>\n#include <time.h>\n")
    s = _sub_once(s, "    i_iter = 0L; error = threshold; save_iter = 0;\n",
                  "    i_iter = 0L; error = threshold; save_iter = 0;\n"
                  "    struct timespec ppf_t0, ppf_t1; clock_gettime(CLOCK_MONOTONIC, &ppf_t0);\n")
    s = _sub_once(s, '    fprintf(STD_BUF,"Total steps: %ld; error: %10.6e\\n",i_iter,error);\n',
                  "    clock_gettime(CLOCK_MONOTONIC, &ppf_t1);\n"
                  '    fprintf(STD_BUF,"ppf-ref loop seconds: %.9f\\n",'
                  " (double)(ppf_t1.tv_sec-ppf_t0.tv_sec)+1e-9*(double)(ppf_t1.tv_nsec-ppf_t0.tv_nsec));\n"
                  '    fprintf(STD_BUF,"Total steps: %ld; error: %10.6e\\n",i_iter,error);\n')
    if omp:
        s = _omp_pragmas(s)
    return s


def tag_of(**kw) -> str:
    key = ",".join(f"{k}={kw[k]}" for k in sorted(kw))
    return hashlib.sha1(key.encode()).hexdigest()[:12]


def build(nz: int, ny: int, nx: int, bc: int = 0, n_iter: int = 1, n_save: int = 1 << 40,
          n_iter_init: int | None = None, dt_expr: str | None = None, fix_etaL: bool = True,
          omp: bool = False, quiet: bool = True) -> str:
    """Build (or reuse) a patched reference binary; returns its path."""
    tag = tag_of(nz=nz, ny=ny, nx=nx, bc=bc, n_iter=n_iter, n_save=n_save, n_iter_init=n_iter_init,
                 dt_expr=dt_expr, fix_etaL=fix_etaL, omp=omp)
    os.makedirs(OUT_DIR, exist_ok=True)
    csrc = os.path.join(OUT_DIR, f"ppf_ref_{tag}.c")
    exe = os.path.join(OUT_DIR, f"ppf_ref_{tag}")
    if os.path.exists(REF_SRC):
        with open(REF_SRC) as f:
            text = patch(f.read(), nz, ny, nx, bc, n_iter, n_save, n_iter_init, dt_expr, fix_etaL, omp)
        old = open(csrc).read() if os.path.exists(csrc) else None
        if old != text:
            with open(csrc, "w") as f:
                f.write(text)
    elif not os.path.exists(csrc):
        raise FileNotFoundError("reference sources absent and no patched unit in oracle/_ref/")
    deps = [csrc, H5REF, os.path.join(SHIM, "h5shim.c"), os.path.join(SHIM, "h5ref.h"), os.path.join(SHIM, "hdf5.h")]
    if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(p) for p in deps):
        return exe
    cmd = ["gcc", "-std=gnu99", "-O2", "-w", "-I", SHIM, csrc, os.path.join(SHIM, "h5shim.c"), H5REF,
           "-o", exe + ".tmp", "-lm"]
    if omp:
        cmd.insert(3, "-fopenmp")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stderr[-4000:])
    os.replace(exe + ".tmp", exe)
    return exe


_LOOP_RE = re.compile(r"ppf-ref loop seconds: ([0-9.eE+-]+)")


def run(exe: str, h5_path: str, threads: int | None = None, timeout: float = 3600) -> dict:
    """Run a reference binary on an input file; returns its stderr lines,
    stdout (output file names) and the timed loop seconds."""
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    # the reference copies argv[1] into char filename[50] (phasefield.c:107,
    # :118): run in the file's directory and pass the bare name
    r = subprocess.run([exe, os.path.basename(h5_path)], capture_output=True, text=True, env=env,
                       timeout=timeout, cwd=os.path.dirname(os.path.abspath(h5_path)))
    m = _LOOP_RE.search(r.stderr)
    return {"rc": r.returncode, "stderr": r.stderr, "stdout": r.stdout,
            "loop_s": float(m.group(1)) if m else None}


def available() -> bool:
    """True when a reference build is possible here (sources or a unit)."""
    return os.path.exists(REF_SRC) or any(
        n.startswith("ppf_ref_") and n.endswith(".c") for n in os.listdir(OUT_DIR)) if os.path.isdir(OUT_DIR) \
        else os.path.exists(REF_SRC)


if __name__ == "__main__":
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--grid", type=int, nargs=3, default=[64, 64, 64], metavar=("NZ", "NY", "NX"))
    ap.add_argument("--bc", type=int, default=0)
    ap.add_argument("--n-iter", type=int, default=1000)
    ap.add_argument("--n-save", type=int, default=1 << 40)
    ap.add_argument("--n-iter-init", type=int, default=None)
    ap.add_argument("--dt", default=None)
    ap.add_argument("--etaL-bug", action="store_true")
    ap.add_argument("--omp", action="store_true")
    a = ap.parse_args()
    print(build(*a.grid, bc=a.bc, n_iter=a.n_iter, n_save=a.n_save, n_iter_init=a.n_iter_init,
                dt_expr=a.dt, fix_etaL=not a.etaL_bug, omp=a.omp))
    sys.exit(0)
