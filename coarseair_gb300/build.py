"""In-tree build of libcair_gpu.so for sm_103a (nvcc, one -gencode, no cmake).

Translation units are compiled in parallel and linked into one shared library next to this
file, where coarseair_gb300._lib loads it.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcair_gpu.so")

# (source, object, extra flags): the API translation unit, and cair_model.cu once per surface
# model so the per-model kernels compile in parallel
SOURCES = [("cair_api.cu", "cair_api.o", []), ("cair_output.cpp", "cair_output.o", []),
           ("cair_stats_host.cpp", "cair_stats_host.o", []), ("cair_sur.cu", "cair_sur.o", []),
           ("cair_sur_probe.cu", "cair_sur_probe.o", []), ("cair_warp.cu", "cair_warp.o", []),
           ("cair_parity.cu", "cair_parity.o", ["-fmad=false"])] + [
    ("cair_model.cu", "cair_model_%s.o" % name, ["-DCAIR_MODEL_ID=%d" % mid])
    for name, mid in (("o3_umn", 1), ("n3_umn", 2), ("o4_umn", 3), ("o3_nn", 4), ("n4_umn", 5), ("o3_bnn", 6),
                      ("n4_pipnn", 7))]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-diag-suppress", "177",
                     "-I", os.path.join(HERE, "..", "include")]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _digest(deps, extra=()):
    """SHA-256 over the sources, the compiler flags and the nvcc version: the library is rebuilt
    whenever this differs from the digest stamped beside it, whatever the files' times."""
    h = hashlib.sha256()
    for d in sorted(deps):
        h.update(os.path.relpath(d, HERE).encode())
        with open(d, "rb") as f:
            h.update(f.read())
    h.update(repr((NVCC_FLAGS, SOURCES, list(extra))).encode())
    try:
        h.update(subprocess.run([nvcc(), "--version"], capture_output=True, text=True).stdout.encode())
    except (OSError, RuntimeError):
        pass
    return h.hexdigest()


STAMP = LIB + ".sha256"


def _stale(deps, extra=()):
    if not os.path.exists(LIB) or not os.path.exists(STAMP):
        return True
    with open(STAMP) as f:
        return f.read().strip() != _digest(deps, extra)


def _deps():
    out = []
    for root, _, files in os.walk(CSRC):
        for f in files:
            if f.endswith((".cu", ".cuh", ".h", ".cpp")):
                out.append(os.path.join(root, f))
    out.append(os.path.join(HERE, "..", "include", "cair_gpu.h"))
    return out


def build(force=False, verbose=False, extra_flags=()):
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    if not force and not _stale(deps, extra_flags):
        if _newer(EXAMPLE, [os.path.join(HERE, "examples", "cair_run.c"), LIB]):
            build_example()
        return LIB
    cc = nvcc()
    objs = []

    def compile_one(entry):
        src, objname, flags = entry
        obj = os.path.join(BUILD, objname)
        cmd = [cc] + NVCC_FLAGS + flags + list(extra_flags) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-4000:]))
        if verbose:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(SOURCES), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(_digest(deps, extra_flags) + "\n")
    build_example()
    return LIB


EXAMPLE = os.path.join(HERE, "examples", "cair_run")


def build_example():
    """The C caller examples/cair_run.c, linked against the library with the host compiler."""
    src = os.path.join(HERE, "examples", "cair_run.c")
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc or not os.path.exists(src):
        return None
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
    cmd = [cc, "-O2", "-std=c11", "-I", os.path.join(HERE, "..", "include"), src, "-o", EXAMPLE, "-L", HERE,
           "-lcair_gpu", "-Wl,-rpath," + HERE, "-L", cuda_lib, "-lcudart", "-Wl,-rpath," + cuda_lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("example build failed:\n" + r.stderr[-4000:])
    return EXAMPLE


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
