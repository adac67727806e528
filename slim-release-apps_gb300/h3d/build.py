"""Build the native parts of h3d in-tree.

* ``libh3d.so``     -- the CUDA library (all of csrc/*.cu), sm_103a only, behind the C ABI
                       declared in include/h3d.h;
* ``h3d_mex/*.so``  -- the drop-in MEX gateways (slim-release-apps_gb300/mex), one per
                       reference binary name, linked against libh3d.so and, for hosting
                       outside MATLAB, the stub MEX API.

Translation units compile in parallel; nothing is rebuilt when outputs are newer than
their sources.  No cmake: plain nvcc/gcc invocations.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
SRC_ROOT = os.path.dirname(PKG)                     # slim-release-apps_gb300/
REPO = os.path.dirname(SRC_ROOT)
CSRC = os.path.join(SRC_ROOT, "csrc")
MEXSRC = os.path.join(SRC_ROOT, "mex")
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libh3d.so")
MEXDIR = os.path.join(LIBDIR, "mex")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]

# The drop-in gateways: reference binary name -> (kind, flags); install_MEX:88-114.
MEX_VARIANTS = {
    "Helm3dmvp_forw_mex": ("mvp", []),
    "Helm3dmvp_forw_wnc_mex": ("mvp", ["-DWNCMPLX"]),
    "Helm3dmvp_forw_deriv_mex": ("mvp", ["-DDERIV"]),
    "Helm3dmvp_adj_mex": ("mvp", ["-DADJ"]),
    "Helm3dmvp_adj_wnc_mex": ("mvp", ["-DADJ", "-DWNCMPLX"]),
    "Helm3dmvp_adj_deriv_mex": ("mvp", ["-DADJ", "-DDERIV"]),
    "Helm3d_kacz_sweep_mex": ("swp", []),
    "Helm3d_kacz_sweep_wnc_mex": ("swp", ["-DWNCMPLX"]),
    "Helm3d_kacz_sweep_adj_mex": ("swp", ["-DADJ"]),
    # the band-storage gateways, install_MEX:75-86
    "Hmvp_MT_mex": ("bmvp", []),
    "sweep_MT_mex": ("bswp", []),
    # the whole linearsolve / CGMN solve in one call (no reference binary of this name)
    "h3d_solve_mex": ("solve", []),
    # FGMRES + ML_GMRES from the physical model in one call (no reference binary of this name)
    "h3d_mlgmres_mex": ("mlgmres", []),
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(out: str, deps) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {' '.join(cmd[:3])} ...")
    return r


class _BuildLock:
    """An exclusive lock file in the output folder: processes that build at the same time
    (ranks of one job) take turns, and the second finds the outputs up to date."""

    def __init__(self):
        os.makedirs(LIBDIR, exist_ok=True)
        self.path = os.path.join(LIBDIR, ".build.lock")
        self.f = None

    def __enter__(self):
        import fcntl

        self.f = open(self.path, "w")
        fcntl.flock(self.f, fcntl.LOCK_EX)
        return self

    def __exit__(self, *exc):
        import fcntl

        fcntl.flock(self.f, fcntl.LOCK_UN)
        self.f.close()


def _compile(cmd_prefix, src, obj, verbose):
    """Compile to a temporary name, then rename: a reader never sees a half-written object."""
    tmp = f"{obj}.{os.getpid()}.tmp"
    _run([*cmd_prefix, "-c", src, "-o", tmp], verbose)
    os.replace(tmp, obj)


def build_lib(verbose: bool = False, force: bool = False, jobs: int | None = None) -> str:
    with _BuildLock():
        return _build_lib(verbose, force, jobs)


def _build_lib(verbose: bool, force: bool, jobs: int | None) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [os.path.join(INCLUDE, "h3d.h")]
    objs = []
    todo = []
    for s in sources:
        o = os.path.join(OBJDIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            todo.append((s, o))
    nv = nvcc()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, [nv, *NVCC_FLAGS], s, o, verbose) for s, o in todo]
        for f in futs:
            f.result()
    if force or todo or not _newer(LIB, objs):
        # link to a temporary name and rename: a process that loads the library meanwhile
        # maps either the old file or the complete new one
        tmp = f"{LIB}.{os.getpid()}.tmp"
        _run([nv, ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs], verbose)
        os.replace(tmp, LIB)
    return LIB


def build_mex(verbose: bool = False, force: bool = False) -> dict:
    """Compile the drop-in gateways against the stub MEX API (oracle/stub) for hosting
    outside MATLAB; inside MATLAB the same source builds with `mex` and the same -D flags."""
    os.makedirs(MEXDIR, exist_ok=True)
    gw = os.path.join(MEXSRC, "h3d_mex_gateway.c")
    stub_dir = os.path.join(REPO, "oracle", "stub")
    stub_c = os.path.join(stub_dir, "mexstub.c")
    out = {}
    cc = shutil.which("gcc") or "cc"
    for name, (kind, flags) in MEX_VARIANTS.items():
        so = os.path.join(MEXDIR, name + ".so")
        out[name] = so
        if not force and _newer(so, [gw, stub_c, LIB, os.path.join(INCLUDE, "h3d.h")]):
            continue
        kflag = {"mvp": "-DH3D_GATEWAY_MVP", "swp": "-DH3D_GATEWAY_SWEEP", "bmvp": "-DH3D_GATEWAY_BAND_MVP",
                 "bswp": "-DH3D_GATEWAY_BAND_SWEEP", "solve": "-DH3D_GATEWAY_SOLVE",
                 "mlgmres": "-DH3D_GATEWAY_MLGMRES"}[kind]
        tmp = f"{so}.{os.getpid()}.tmp"
        _run([cc, "-O2", "-std=c11", "-fPIC", "-shared", kflag, *flags, "-I", INCLUDE, "-I",
              stub_dir, gw, stub_c, "-o", tmp, "-L", LIBDIR, "-lh3d",
              "-Wl,-rpath,$ORIGIN/.."], verbose)
        os.replace(tmp, so)
    return out


def build(verbose: bool = False, force: bool = False) -> str:
    lib = build_lib(verbose=verbose, force=force)
    if os.path.exists(os.path.join(MEXSRC, "h3d_mex_gateway.c")):
        with _BuildLock():
            build_mex(verbose=verbose, force=force)
    return lib


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
