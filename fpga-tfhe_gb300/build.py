"""Build recipe of the engine: nvcc, sm_103a only, in-tree.

Compiles fpga-tfhe_gb300/csrc/*.cu and *.cpp in parallel into objects under
fpga-tfhe_gb300/_build/ and links fpga-tfhe_gb300/libtfhe_gb300.so (CUDA
runtime linked statically, so the library has no runtime dependency beyond
the driver).  No cmake; a rebuild only recompiles changed translation units.

    python fpga-tfhe_gb300/build.py [--force] [--verbose]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtfhe_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-Wall,-Wno-unknown-pragmas",
          "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    for d in (INCLUDE, os.path.join(INCLUDE, "tfhe")):
        hs += [os.path.join(d, f) for f in os.listdir(d) if f.endswith(".h")]
    return hs


def _obj(src):
    return os.path.join(BUILD, os.path.basename(src) + ".o")


def _compile(src, verbose, extra):
    obj = _obj(src)
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force=False, verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    newest_hdr = max(os.path.getmtime(h) for h in _headers())
    todo = [s for s in srcs if force or ptxas_info or not os.path.exists(_obj(s))
            or os.path.getmtime(_obj(s)) < max(os.path.getmtime(s), newest_hdr)]
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    logs = []
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(todo))) as ex:
            for log in ex.map(lambda s: _compile(s, verbose, extra), todo):
                logs.append(log)
    if todo or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + [_obj(s) for s in srcs]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    if ptxas_info:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv,
                ptxas_info="--ptxas" in sys.argv))
