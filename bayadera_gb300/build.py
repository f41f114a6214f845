"""Builds libbayadera_gb300.so in-tree with nvcc (sm_103a only).

The device sources that NVRTC compiles at model-compile time (csrc/device/*.cuh)
are embedded into the library as string literals, so the shared object is
self-contained: a host binding needs only the .so and include/bayadera_gb300.h.
"""
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(CSRC, "_build")
LIB = os.path.join(PKG, "libbayadera_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]

EMBED = [("bay_embedded_rng", "device/bay_rng.cuh"),
         ("bay_embedded_stretch", "device/bay_stretch.cuh"),
         ("bay_embedded_batch", "device/bay_batch.cuh"),
         ("bay_embedded_direct", "device/bay_direct.cuh"),
         ("bay_embedded_hist_fastdiv", "device/bay_hist_fastdiv.cuh")]
SOURCES = ["bay_api.cpp", "bay_kernels.cu"]
HEADERS = ["bay_kernels.cuh", "bay_batch_api.inc", "bay_engines_api.inc", "bay_tune_api.inc",
           os.path.join("..", "..", "include", "bayadera_gb300.h")]


def cuda_home():
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for c in ("/usr/local/cuda", "/usr/local/cuda-13.0"):
        if os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build bayadera_gb300")


def _write_embedded():
    os.makedirs(BUILD, exist_ok=True)
    out = ["// generated by bayadera_gb300/build.py -- device sources for NVRTC", "#pragma once"]
    for name, rel in EMBED:
        with open(os.path.join(CSRC, rel)) as f:
            text = "".join(l for l in f if l.strip() != "#pragma once")
        if ")BAYSRC\"" in text:
            raise RuntimeError("delimiter clash in " + rel)
        out.append('static const char* %s = R"BAYSRC(%s)BAYSRC";' % (name, text))
    path = os.path.join(BUILD, "bay_embedded.h")
    data = "\n".join(out) + "\n"
    if not os.path.exists(path) or open(path).read() != data:
        with open(path, "w") as f:
            f.write(data)
    return path


def _inputs():
    files = [os.path.join(CSRC, s) for s in SOURCES] + [os.path.join(CSRC, h) for h in HEADERS]
    files += [os.path.join(CSRC, rel) for _, rel in EMBED]
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _inputs())


def build(force=False, verbose=False):
    """Compile the library if any input is newer than it.  Returns the .so path."""
    if not force and up_to_date():
        return LIB
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    _write_embedded()
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + BUILD]
    procs = []
    objs = []
    for s in SOURCES:
        obj = os.path.join(BUILD, os.path.splitext(s)[0] + ".o")
        objs.append(obj)
        cmd = [nvcc] + ARCH + NVCC_FLAGS + inc + ["-c", os.path.join(CSRC, s), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out.decode()))
        if verbose and out:
            print(out.decode())
    lib64 = os.path.join(home, "lib64")
    tmp = LIB + ".tmp"
    link = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + [
        "-L" + lib64, "-lnvrtc",
        "-Xlinker", "-rpath," + lib64]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (" ".join(link), r.stdout.decode()))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
