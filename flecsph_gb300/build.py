"""Build libfsph_gb300.so in-tree with nvcc for sm_103a.

    python -m flecsph_gb300.build          # or flecsph_gb300.build.build()

Translation units that must round like the reference's FP64 code (keys,
neighbour predicate, plain-FP64 physics, integrator) are compiled with
-fmad=false; the mixed-precision kernels may contract.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfsph_gb300.so")
DRIVER = os.path.join(HERE, "hydro_driver")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = {
    "fsph_tree.cu": ["-fmad=false"],
    "fsph_fp64.cu": ["-fmad=false"],
    "fsph_elementwise.cu": ["-fmad=false"],
    "fsph_mixed.cu": ["-prec-div=false", "-prec-sqrt=false"],
    "fsph_mixed_cullen.cu": ["-prec-div=false", "-prec-sqrt=false"],
    "fsph_gravity.cu": [],
    "fsph_periodic.cu": ["-fmad=false"],
    "fsph_peak.cu": [],
    "fsph_api.cu": [],
    "fsph_ensemble.cu": [],
}


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _tuning_defines():
    """-D flags from $FSPH_NVCC_DEFINES ("NAME=VALUE NAME2=VALUE2"): launch-shape
    knobs of the kernels (FSPH_ACCEL_FF_BLOCKS, NB_UNI_BLOCKS_PER_SM, RS_ITEMS,
    ...), for tuning runs; empty for
    the default build."""
    return ["-D" + d for d in os.environ.get("FSPH_NVCC_DEFINES", "").split() if d]


def _compile(src, extra, verbose):
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xptxas", "-v" if verbose else "-O3", *_tuning_defines(), *extra, "-c",
           os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj, r.stderr


def _stale(objs):
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "fsph.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile every CUDA source and link the shared library (in-tree)."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if not force and not _stale(srcs):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        futs = [ex.submit(_compile, s, SOURCES[s], verbose) for s in srcs]
        res = [f.result() for f in futs]
    if verbose:
        for _, log in res:
            sys.stderr.write(log)
    objs = [o for o, _ in res]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver()
    return LIB


def build_driver():
    """The C++ hydro driver (csrc/hydro_driver.cpp) over the C ABI."""
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", os.path.join(CSRC, "hydro_driver.cpp"),
           "-L" + HERE, "-lfsph_gb300", "-Wl,-rpath,$ORIGIN", "-o", DRIVER]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stderr}")
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
