"""In-tree build of libpolyred_cuda.so for GB300 (sm_103a).

Three translation units compiled in parallel:
  csrc/pr_kernels.cu   nvcc, -gencode arch=compute_103a,code=sm_103a, with
                       -fmad=false -prec-div=true -prec-sqrt=true -ftz=false
                       (the render path needs the reference's exact float32
                       roundings: no contraction, IEEE division/sqrt, denormals)
  csrc/pr_api.cpp      host C++, -ffp-contract=off
  csrc/pr_hostmath.cpp host C++, -ffp-contract=off
and linked with the static CUDA runtime into polyred_gb300/lib/.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
BUILD = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(LIBDIR, "libpolyred_cuda.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-ftz=false", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function"]


def cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cpp", ".cuh", ".h"))] + [os.path.join(HERE, "..", "include", h)
                                                             for h in ("polyred_cuda.h", "polyred_cuda_testing.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in sources())


def build(force=False, verbose=False):
    """Compile the library if any source is newer than it; return its path."""
    if not force and up_to_date():
        return LIB
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + os.path.join(cuda, "include"), "-I" + CSRC]
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    objs = []
    for src in sorted(os.listdir(CSRC)):
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        if src.endswith(".cu"):
            cmd = [nvcc] + ARCH + NVCC_FLAGS + inc + ["-c", path, "-o", obj]
        elif src.endswith(".cpp"):
            cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + inc + ["-c", path, "-o", obj]
        else:
            continue
        objs.append(obj)
        jobs.append((src, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, cmd, proc in jobs:
        out, _ = proc.communicate()
        log = os.path.join(BUILD, src + ".log")
        with open(log, "w") as f:
            f.write(" ".join(cmd) + "\n" + out)
        if proc.returncode != 0:
            failed.append((src, out))
        elif verbose:
            sys.stdout.write(out)
    if failed:
        msg = "\n".join(f"--- {s} ---\n{o}" for s, o in failed)
        raise RuntimeError("libpolyred_cuda build failed:\n" + msg)
    tmp = LIB + ".tmp"
    link = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
