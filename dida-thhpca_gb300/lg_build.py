"""Build the LETKF CUDA library in-tree: _build/libletkf_gb300.so (sm_103a only).

Each translation unit is compiled in parallel with nvcc; host code gets
-ffp-contract=off (the neighbour-block distances are REAL(4) expressions whose
rounding must not change by fusion, which matters on aarch64 where the host
compiler would otherwise fuse), and the H(x) / selection kernels get
-fmad=false for the same reason on the device.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libletkf_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                 "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
UNITS = {
    "lg_api.cu": [],
    "lg_hx.cu": ["-fmad=false"],
    "lg_search.cu": ["-fmad=false"],
    "lg_gram.cu": [],
    "lg_eig.cu": [],
    "lg_gram_tc.cu": [],
    "lg_gram_tc128.cu": [],
    "lg_gram_tf32.cu": [],
    "lg_gram_col.cu": [],
    "lg_eig2.cu": [],
    "lg_noalloc.cu": [],
    "lg_prepost.cu": [],
    "lg_cube.cu": [],
    "lg_coupler.cu": [],
}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [
        os.path.join(HERE, "..", "include", "letkf_gpu.h"), os.path.abspath(__file__)]
    newest = max(os.path.getmtime(p) for p in deps)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > newest:
        return LIB
    nvcc = _nvcc()

    def compile_one(name):
        obj = os.path.join(OUT, name.replace(".cu", ".o"))
        cmd = [nvcc] + COMMON + UNITS[name] + ["-c", os.path.join(SRC, name), "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(compile_one, UNITS))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
