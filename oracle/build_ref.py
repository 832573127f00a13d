"""Builds oracle/_ref/libwfref.so: the reference's own kernel sources compiled
for the CPU, used only to pin the oracle (test infrastructure).

The sources are read where they lie in the reference tree: $WF_REFERENCE_DIR,
or else a directory named `reference` beside the repository's root; nothing is
copied.  The reference's
CMake build is not used: two translation units written here
(ref_domain.cpp, ref_nsearch.cpp) #include the reference's kernel files, and
cuda_host_shim.h stands in for the CUDA built-ins.  Flags keep IEEE
semantics (-ffp-contract=off), like the reference's --fmad=false.

Usage: python oracle/build_ref.py   (no-op when the reference tree is absent)
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "libwfref.so")


def reference_dir():
    """$WF_REFERENCE_DIR, else `reference` beside the repository's root."""
    env = os.environ.get("WF_REFERENCE_DIR")
    if env:
        return env
    return os.path.normpath(os.path.join(HERE, "..", "..", "reference"))


# Thermal.cu's kernels, taken verbatim: the file also holds host functions that
# launch kernels with <<< >>>, which g++ cannot parse, so only these functions
# are written into the build directory for ref_domain.cpp to #include.
THERMAL_KERNELS = ("TempCalcLeapfrogFirst", "TempCalcLeapfrog", "CalcConvHeatKernel",
                   "ThermalSolveKernel")


def extract_kernels(path, names):
    """The text of each `__global__` function definition named in `names` (the
    overload whose parameter list is not a single PartData_d pointer), from
    its start line to its matching closing brace."""
    text = open(path).read()
    out = []
    for name in names:
        pos = 0
        found = False
        while True:
            k = text.find(name, pos)
            if k < 0:
                break
            pos = k + len(name)
            line_start = text.rfind("\n", 0, k) + 1
            head = text[line_start:k]
            if "__global__" not in head or text[pos:].lstrip()[:1] != "(":
                continue
            brace = text.find("{", pos)
            semi = text.find(";", pos)
            if brace < 0 or (0 <= semi < brace):        # a declaration, not a definition
                continue
            if "PartData_d" in text[pos:brace]:
                continue
            depth, q = 0, brace
            while True:
                if text[q] == "{":
                    depth += 1
                elif text[q] == "}":
                    depth -= 1
                    if depth == 0:
                        break
                q += 1
            out.append(text[line_start:q + 1])
            found = True
            break
        if not found:
            raise RuntimeError("kernel %s not found in %s" % (name, path))
    return "namespace SPH {\n" + "\n\n".join(out) + "\n}  // namespace SPH\n"


def build(verbose=False):
    ref = reference_dir()
    src = os.path.join(ref, "src")
    if not os.path.isdir(os.path.join(src, "cuda")):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    with open(os.path.join(OUT_DIR, "thermal_kernels.inc"), "w") as f:
        f.write(extract_kernels(os.path.join(src, "cuda", "Thermal.cu"), THERMAL_KERNELS))
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    inc = [
        "-I" + OUT_DIR,
        "-I" + os.path.join(HERE, "ref_shim"),
        "-I" + os.path.join(src, "cuda"),
        "-I" + src,
        "-I" + os.path.join(src, "cuNSearch", "include"),
        "-I" + os.path.join(src, "cuNSearch", "src"),
        "-I" + os.path.join(src, "cuNSearch", "Utils"),
        "-I" + os.path.join(cuda, "include"),
        "-I" + os.path.join(cuda, "include", "cccl"),
    ]
    flags = ["-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-w",
             "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP", "-Wno-cpp"]
    objs = []
    for tu in ("ref_domain.cpp", "ref_nsearch.cpp", "ref_nastran.cpp"):
        obj = os.path.join(OUT_DIR, tu.replace(".cpp", ".o"))
        cmd = ["g++"] + flags + inc + ["-c", os.path.join(HERE, tu), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("building %s failed:\n%s" % (tu, r.stderr))
        objs.append(obj)
    subprocess.run(["g++", "-shared", "-o", OUT] + objs + ["-lm"], check=True)
    return OUT


if __name__ == "__main__":
    out = build(verbose="-v" in sys.argv)
    print(out or "reference tree not found: oracle/_ref not built")
