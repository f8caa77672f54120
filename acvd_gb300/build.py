"""Builds the CUDA library libacvd_gb300.so in-tree (acvd_gb300/_build/) for sm_103a.

    python -m acvd_gb300.build        # or acvd_gb300.build.build()

Each translation unit is compiled by nvcc in parallel; the link is a plain
`nvcc -shared`.  No CMake, no torch extension machinery: the library exposes a
C ABI (include/acvd_gpu.h) and is loaded with ctypes.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libacvd_gb300.so")
# the plain float32 form: cluster.cu compiled with ACVD_PLAIN_FP32 (uncompensated
# cluster sums), linked with the other objects into a second library
LIB_PLAIN = os.path.join(OUT, "libacvd_gb300_plain.so")
PLAIN_SOURCE = "cluster.cu"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CU_SOURCES = ["primitives.cu", "topology.cu", "cluster.cu", "adjoint.cu", "engine.cu", "noalloc.cu", "curvature.cu", "subdivide.cu",
              "manifold.cu"]
# per-file flags: the curvature kernel keeps every FP64 product and sum separately
# rounded, so that it reproduces the CPU restatement bit for bit
CU_FILE_FLAGS = {"curvature.cu": ["-fmad=false"]}
CXX_SOURCES = ["host.cpp", "io.cpp"]
# command-line programs built from csrc/acvd_cli.cpp: name -> compile definitions
CLI_PROGRAMS = {"acvd": [], "acvdq": ["-DACVD_CLI_QEM"], "anisotropic_remeshing_q": ["-DACVD_CLI_ANISO"]}


# the libtorch autograd function over acvd_adjoint_on_stream (csrc/adjoint_torch.cpp),
# compiled by torch.utils.cpp_extension into _build/torch_ext
TORCH_EXT_NAME = "acvd_adjoint_torch"
TORCH_EXT_DIR = os.path.join(OUT, "torch_ext")


def load_torch_extension(verbose: bool = False):
    """Builds (when stale) and imports the libtorch extension module."""
    from torch.utils import cpp_extension
    os.makedirs(TORCH_EXT_DIR, exist_ok=True)
    return cpp_extension.load(name=TORCH_EXT_NAME, sources=[os.path.join(SRC, "adjoint_torch.cpp")],
                              extra_cflags=["-O2", "-std=c++17"], with_cuda=True, build_directory=TORCH_EXT_DIR,
                              verbose=verbose)


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """ACVD_NVCC_FLAGS (environment) adds nvcc flags (e.g. -DACVD_DEVICE_CHECKS for the
    self-checking build); pass force=True (or --force) when they change.  The evaluation
    kernels' blocks per SM are a run-time choice (ACVD_EVAL_BLOCKS), not a build flag."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    extra = os.environ.get("ACVD_NVCC_FLAGS", "").split()
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "acvd_gpu.h"))
    jobs = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "-diag-suppress", "128"] + CU_FILE_FLAGS.get(f, []) + extra + ["-c", src, "-o", obj])
    plain_obj = os.path.join(OUT, "cluster_plain.cu.o")
    src = os.path.join(SRC, PLAIN_SOURCE)
    if force or _stale(plain_obj, [src] + headers):
        jobs.append([nvcc, ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-diag-suppress", "128", "-DACVD_PLAIN_FP32"] + extra + ["-c", src, "-o", plain_obj])
    for f in CXX_SOURCES:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            # no FMA contraction: the host arithmetic gives the same bits on x86 and Arm
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    # the native ACVD / ACVDQ programs over the C ABI
    cli_src = os.path.join(SRC, "acvd_cli.cpp")
    cli_jobs = []
    for name, defs in CLI_PROGRAMS.items():
        obj = os.path.join(OUT, name + ".o")
        if force or _stale(obj, [cli_src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-ffp-contract=off"] + defs + ["-c", cli_src, "-o", obj])
            cli_jobs.append(name)

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(jobs)) + 1) as ex:
        torch_ext = ex.submit(load_torch_extension, verbose)   # in parallel with the nvcc jobs
        list(ex.map(run, jobs))
        torch_ext.result()
    relinked = force or bool(jobs) or not os.path.exists(LIB) or not os.path.exists(LIB_PLAIN)
    if relinked:
        run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart"])
        plain_objs = [plain_obj if o.endswith(os.sep + PLAIN_SOURCE + ".o") else o for o in objs]
        run([nvcc, ARCH, "-shared", "-o", LIB_PLAIN] + plain_objs + ["-lcudart"])
    for name in CLI_PROGRAMS:
        exe = os.path.join(OUT, name)
        if relinked or name in cli_jobs or not os.path.exists(exe):
            run(["g++", "-o", exe, os.path.join(OUT, name + ".o"), "-L" + OUT, "-lacvd_gb300",
                 "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="--force" in sys.argv))
