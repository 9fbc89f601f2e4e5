"""Builds libfalcon_gpu.so (sm_103a) in-tree under falcon-dns_gb300/_build/.

The CUDA translation units (nvcc, -gencode arch=compute_103a,code=sm_103a)
and the host runtime (g++) compile in parallel and are linked with nvcc;
then the namelist-driven executable falcon_run (driver/falcon_run.cpp,
C ABI only) is linked against the library.  Host code is compiled with -ffp-contract=off so that
operator construction gives identical results on x86_64 and aarch64.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfalcon_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), nvcc


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("build step failed: " + cmd[0])
    return r.stdout + r.stderr


DRIVER_SRC = os.path.join(HERE, "driver", "falcon_run.cpp")
DRIVER = os.path.join(OUT, "falcon_run")


def sources():
    return [os.path.join(SRC, f) for f in sorted(os.listdir(SRC))] + [
        os.path.join(HERE, "..", "include", "falcon_gpu.h"), DRIVER_SRC]


def up_to_date():
    if not os.path.exists(LIB) or not os.path.exists(DRIVER):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(DRIVER))
    return all(os.path.getmtime(s) <= t for s in sources())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    home, nvcc = _cuda_home()
    cu_srcs = sorted(f for f in os.listdir(SRC) if f.endswith(".cu"))
    objs = [os.path.join(OUT, f[:-3] + ".o") for f in cu_srcs]
    host_o = os.path.join(OUT, "falcon_host.o")
    cmds = [[nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
                             "-c", os.path.join(SRC, f), "-o", o] for f, o in zip(cu_srcs, objs)]
    cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
                 "-I" + os.path.join(home, "include"), "-c", os.path.join(SRC, "falcon_host.cpp"), "-o", host_o])
    with ThreadPoolExecutor(len(cmds)) as ex:
        logs = list(ex.map(_run, cmds))
    if verbose:
        print(logs[0])
    tmp = LIB + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + [host_o, "-lcudart", "-lpthread"])
    os.replace(tmp, LIB)
    # the namelist-driven executable (C ABI only), next to the library
    _run(["g++", "-O2", "-std=c++17", DRIVER_SRC, "-o", DRIVER + ".tmp", "-L" + OUT, "-lfalcon_gpu",
          "-Wl,-rpath,$ORIGIN"])
    os.replace(DRIVER + ".tmp", DRIVER)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
