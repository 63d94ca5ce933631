"""Build recipe for libpychem_gb300.so (sm_103a only, no CMake).

Every .cu file under csrc/ is compiled to an object in parallel with nvcc and
linked into pychem_gb300/libpychem_gb300.so next to this file (in-tree, git-ignored).
Objects are rebuilt when a source or any header in csrc/ or include/ is newer.

    python -m pychem_gb300.build
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpychem_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     "--expt-relaxed-constexpr"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build pychem_gb300")
    return path


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _regen_if_stale():
    gen = os.path.join(CSRC, "gen_eri.py")
    out = os.path.join(CSRC, "eri_gen.cuh")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(gen):
        subprocess.check_call([sys.executable, gen], stdout=subprocess.DEVNULL)


def build(verbose=False, jobs=None):
    _regen_if_stale()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_time = _newest_header()
    todo = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_time):
            todo.append((s, o))
    # largest translation units first
    todo.sort(key=lambda so: -os.path.getsize(so[0]) - (10 ** 9 if "eri_g" in so[0] else 0))

    def compile_one(so):
        s, o = so
        cmd = [nvcc()] + NVCC_FLAGS + ["-I" + CSRC, "-I" + INCLUDE, "-c", s, "-o", o + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s" % (s, r.stderr[-4000:]))
        os.replace(o + ".tmp", o)
        if verbose:
            print("compiled", os.path.basename(s), flush=True)

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(compile_one, todo))
    if todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread",
                                                                 "-Xlinker", "-rpath=" + os.path.join(CUDA_HOME, "lib64")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
        os.replace(LIB + ".tmp", LIB)
        if verbose:
            print("linked", LIB, flush=True)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
