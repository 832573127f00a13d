"""Builds libweldform_gb300.so in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel; the FP64 step and integration
units use -fmad=false so that multiplies and adds round separately, as in the
reference build (--fmad=false, src/CMakeLists.txt:29).  No torch, no cmake.

Usage: python -m weldformgpu_gb300.build [-v] [--force]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libweldform_gb300.so")
CLI = os.path.join(HERE, "wf")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "--expt-relaxed-constexpr"]
# units whose FP64 arithmetic must round like the reference / the CPU oracle
NO_FMA = {"wf_step_fp64.cu", "wf_integrate.cu", "wf_contact.cu", "wf_outputs.cu"}
SOURCES = ["wf_api.cu", "wf_nsearch.cu", "wf_step_fp64.cu", "wf_step_fp32.cu", "wf_integrate.cu",
           "wf_mlp.cu", "wf_setup.cpp", "wf_noalloc.cu", "wf_contact.cu", "wf_json.cpp",
           "wf_outputs.cu", "wf_measure.cu", "wf_tiles.cu"]


def nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "weldform_gb300.h"))
    return max(os.path.getmtime(f) for f in files)


def up_to_date():
    return (os.path.exists(LIB) and os.path.exists(CLI)
            and min(os.path.getmtime(LIB), os.path.getmtime(CLI)) >= _deps())


def _compile(src, verbose):
    obj = os.path.join(BUILD, src + ".o")
    flags = list(COMMON)
    if src in NO_FMA:
        flags.append("-fmad=false")
    cmd = [nvcc()] + ARCH + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    return obj


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    # the command-line driver (wf <input.json> [out dir]), linked to the library
    cli = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-o", CLI,
           os.path.join(CSRC, "wf_cli.cpp"), "-L" + HERE, "-lweldform_gb300",
           "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cli), flush=True)
    subprocess.run(cli, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
