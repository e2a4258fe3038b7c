"""Builds libltpg.so, the C-ABI engine, from ltpg_gb300/csrc for sm_103a, and
libltpg_bench.so, the measurement-only library, from ltpg_gb300/csrc/bench.

Each translation unit is compiled by its own nvcc process in parallel, then the
objects are linked into ltpg_gb300/libltpg.so (and libltpg_bench.so).  Objects
go to ltpg_gb300/_build.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libltpg.so")
BENCH_CSRC = os.path.join(CSRC, "bench")
BENCH_LIB = os.path.join(HERE, "libltpg_bench.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(HERE, "..", "include")]
# the device generator's double arithmetic must round like the host's: no
# contraction into fused multiply-adds
EXTRA = {"gen_dev.cu": ["-fmad=false"]}


def nvcc():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(home, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _bench_sources():
    return sorted(os.path.join("bench", f) for f in os.listdir(BENCH_CSRC) if f.endswith(".cu"))


def _compile(src):
    obj = os.path.join(BUILD, src.replace(os.sep, "_") + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *EXTRA.get(src, []), "-lineinfo", "--expt-relaxed-constexpr", "-c",
           os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB) or not os.path.exists(BENCH_LIB):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(BENCH_LIB))
    inputs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    inputs += [os.path.join(BENCH_CSRC, f) for f in os.listdir(BENCH_CSRC)]
    inputs += [os.path.join(HERE, "..", "include", h) for h in ("ltpg.h", "ltpg_bench.h")]
    inputs.append(os.path.abspath(__file__))
    return any(os.path.getmtime(p) > t for p in inputs)


def _link(objs, out):
    tmp = out + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of {os.path.basename(out)} failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)


def build(force=False, verbose=False):
    """Compile and link libltpg.so if any source is newer than it; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs, bench = _sources(), _bench_sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs) + len(bench))) as ex:
        results = list(ex.map(_compile, srcs + bench))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    _link(objs[:len(srcs)], LIB)
    _link(objs[len(srcs):], BENCH_LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
