"""Build the CUDA library in-tree: molflow_sources_gb300/_build/libmfg.so (sm_103a).

Six translation units compiled in parallel with nvcc (the kernels + C ABI as
CUDA; the host-side model builder, the XML/ZIP reader and writer and the
results comparison as plain C++), linked with the static CUDA runtime.  No cmake.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmfg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "model_build.cpp", "xml_file.cpp", "xml_model.cpp", "xml_writer.cpp", "compare.cpp"]
DEPS = SOURCES + ["trace_kernels.cuh", "traversal.cuh", "philox.cuh", "anglemap_gen.cuh", "device_model.h",
                  "model_build.h", "xml_file.h", "xml_model.h", "xml_writer.h", "compare.h"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    inc = os.path.join(os.path.dirname(HERE), "include", "mfg.h")
    return any(os.path.getmtime(os.path.join(CSRC, f)) > t for f in DEPS) or os.path.getmtime(inc) > t


def build(force=False, verbose=False):
    """Compile libmfg.so when a source is newer than it; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo"]
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src.replace(".", "_") + ".o")
        objs.append(obj)
        cmd = [nvcc()] + ARCH + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cu"):
            cmd += ["-split-compile=0"]   # the kernel variants are optimised on all host cores
            cmd += ["-Xptxas", "-v"] if verbose else []
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(out.decode(errors="replace"))
        crashed = p.returncode < 0 or p.returncode in (134, 139) or b"Segmentation fault" in out or b"core dumped" in out
        if p.returncode and crashed:
            # the compiler itself crashed (a signal, not a diagnostic): once more on one thread, then
            # with the node fetches as two 16-byte loads (MFG_NO_V8), the form every toolchain takes
            retries = ([c for c in cmd if c != "-split-compile=0"],
                       [c for c in cmd if c != "-split-compile=0"] + ["-DMFG_NO_V8"])
            for again in retries:
                sys.stderr.write("compiler crashed (status %d); retrying: %s\n" % (p.returncode, " ".join(again)))
                r = subprocess.run(again, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
                if r.returncode == 0:
                    break
                sys.stderr.write(r.stdout.decode(errors="replace"))
            else:
                raise RuntimeError("compile failed: " + " ".join(cmd))
            continue
        if p.returncode:
            raise RuntimeError("compile failed: " + " ".join(cmd))
    tmp = LIB + ".tmp%d" % os.getpid()
    link = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs + ["-lpthread"]
    subprocess.run(link, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
