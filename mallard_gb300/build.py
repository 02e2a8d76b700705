"""In-tree build of libmallard_gb300.so (CUDA kernels for sm_103a + host C++).

    python -m mallard_gb300.build          # incremental
    python -m mallard_gb300.build --force

Objects and the library go to mallard_gb300/_build/ (git-ignored).  The
kernels are compiled with -fmad=false: the FP64 path keeps the reference's
rounding (no contraction of a*b+c).  Host code uses -ffp-contract=off for the
same reason, which also keeps x86 and aarch64 hosts bit-identical.
"""

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libmallard_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and Path(cand, "bin", "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _sources():
    cu = sorted(SRC.glob("*.cu"))
    cpp = sorted(SRC.glob("*.cpp"))
    headers = sorted(SRC.glob("*.h")) + sorted(SRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    return cu, cpp, headers


def _jobs(cuda):
    nvcc = str(cuda / "bin" / "nvcc")
    inc = f"-I{cuda / 'include'}"
    cu, cpp, _ = _sources()
    jobs = []
    for s in cu:
        o = OUT / (s.stem + ".o")
        # *_fast.cu may contract a*b+c into FMA; everything else keeps two roundings
        fmad = "-fmad=true" if s.stem.endswith("_fast") else "-fmad=false"
        # the stencil search calls std::sort in device code: constexpr (and
        # so callable there) from C++20 on
        std = ["-std=c++20", "--expt-relaxed-constexpr"] if s.stem == "stencil_search" else ["-std=c++17"]
        jobs.append((o, [nvcc, ARCH, "-O3", "-lineinfo", fmad, *std, "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v", "-c", str(s), "-o", str(o)]))
    cxx = os.environ.get("CXX", "g++")
    for s in cpp:
        o = OUT / (s.stem + ".o")
        jobs.append((o, [cxx, "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
                         "-Wall", "-Wextra", inc, "-c", str(s), "-o", str(o)]))
    return jobs


def build(force=False, verbose=False):
    """Compile every extension source; returns the library path."""
    cuda = cuda_home()
    OUT.mkdir(parents=True, exist_ok=True)
    cu, cpp, headers = _sources()
    newest_src = max(p.stat().st_mtime for p in cu + cpp + headers + [Path(__file__)])
    if not force and LIB.exists() and LIB.stat().st_mtime > newest_src:
        return LIB
    procs = []
    for obj, cmd in _jobs(cuda):
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((obj, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    logs = []
    for obj, cmd, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        logs.append((obj.name, text))
        if p.returncode != 0:
            failed.append((obj, cmd, text))
    (OUT / "ptxas.log").write_text("".join(f"== {n}\n{t}\n" for n, t in logs))
    if failed:
        msg = "\n".join(f"$ {' '.join(c)}\n{t}" for _, c, t in failed)
        raise RuntimeError(f"mallard_gb300 build failed:\n{msg}")
    objs = [str(o) for o, _ in _jobs(cuda)]
    tmp = LIB.with_suffix(".so.tmp")
    link = [os.environ.get("CXX", "g++"), "-shared", "-fopenmp", "-o", str(tmp)] + objs + [
        f"-L{cuda / 'lib64'}", f"-Wl,-rpath,{cuda / 'lib64'}", "-lcudart"]
    if verbose:
        print(" ".join(link), flush=True)
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
