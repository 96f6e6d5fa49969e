"""Build recipe for the solver library (``lib/librfmm.so``).

Compiles every translation unit under ``csrc/`` with nvcc for sm_103a only,
in parallel, and links one shared library exporting the C ABI declared in
``include/rainbow_fmm.h`` and ``include/rfmm.h``.

Kernel translation units are compiled with ``-fmad=false`` and IEEE division
and square root, which is the floating-point contract the kernels rely on to
match the CPU oracle bit for bit.  The tree and body kernels are compiled a
second time with ``-DRFMM_FAST_FLOAT`` (namespace ``rfmm::fast``), contraction
on, approximate division and square root and subnormals flushed to zero: the
fast float variant.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # fmm-rainbow_gb300/
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "librfmm.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", CSRC, "-I", INCLUDE,
          "-I", BUILD]
KERNEL_FLAGS = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
FAST_FLAGS = ["-DRFMM_FAST_FLOAT", "-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
# Compiled again in the fast float variant (object name, source).
FAST_SOURCES = ["kernels_tree.cu", "kernels_body.cu"]

SOURCES = [
    "kernels_tree.cu",
    "kernels_body.cu",
    "kernels_sort.cu",
    "kernels_diag.cu",
    "kernels_render.cu",
    "noalloc.cu",
    "engine.cpp",
    "capi.cpp",
    "capi_batch.cpp",
    "server.cpp",
    "planner.cpp",
]
# Text embedded as the "shader" payload of rainbow_shader_ptr().
EMBEDDED = ["rfmm_device.cuh", "kernels_tree.cu", "kernels_body.cu", "kernels_sort.cu"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _gen_source_text() -> str:
    os.makedirs(BUILD, exist_ok=True)
    text = b""
    for name in EMBEDDED:
        with open(os.path.join(CSRC, name), "rb") as f:
            text += b"// ---- " + name.encode() + b"\n" + f.read() + b"\n"
    body = ",".join(str(b) for b in text)
    out = os.path.join(BUILD, "kernel_source.cpp")
    src = (
        "// Generated by build.py: CUDA source text of the solver kernels.\n"
        "#include <cstddef>\n#include \"rfmm_internal.h\"\n"
        "namespace rfmm {\nnamespace {\nconst char kText[] = {%s, 0};\n}\n"
        "const char *kernel_source_text() { return kText; }\n"
        "size_t kernel_source_len() { return sizeof(kText) - 1; }\n}\n" % body
    )
    old = open(out).read() if os.path.exists(out) else None
    if old != src:
        with open(out, "w") as f:
            f.write(src)
    return out


def _compile(src: str, obj: str, extra=(), fast: bool = False) -> None:
    flags = list(COMMON) + list(ARCH) + list(extra)
    if src.endswith(".cu"):
        flags += FAST_FLAGS if fast else KERNEL_FLAGS
    cmd = [nvcc(), *flags, "-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), res.stderr))


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return files + [os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, csrc: str | None = None, lib: str | None = None,
          extra_flags=()) -> str:
    """Compile and link ``lib/librfmm.so`` if any input changed.

    ``csrc``/``lib``/``extra_flags`` build an alternative source tree into an
    alternative library path (used to compare kernel variants side by side).
    """
    if csrc is None and lib is None and not extra_flags:
        if not force and up_to_date():
            return LIB
        csrc_dir, out_lib, build_dir = CSRC, LIB, BUILD
    else:
        csrc_dir = csrc or CSRC
        out_lib = lib or LIB
        build_dir = os.path.join(os.path.dirname(os.path.abspath(out_lib)), "_build")
    os.makedirs(build_dir, exist_ok=True)
    os.makedirs(os.path.dirname(os.path.abspath(out_lib)), exist_ok=True)
    srcs = [os.path.join(csrc_dir, s) for s in SOURCES] + [_gen_source_text()]
    objs = [os.path.join(build_dir, os.path.basename(s) + ".o") for s in srcs]
    jobs = [(s, o, False) for s, o in zip(srcs, objs)]
    for f in FAST_SOURCES:
        o = os.path.join(build_dir, f + ".fast.o")
        jobs.append((os.path.join(csrc_dir, f), o, True))
        objs.append(o)
    extra = list(extra_flags) + ["-I", csrc_dir]
    # The largest translation units first, so they start before the short ones.
    jobs.sort(key=lambda j: -os.path.getsize(j[0]))
    with cf.ThreadPoolExecutor(max_workers=min(os.cpu_count() or 8, len(jobs))) as ex:
        list(ex.map(lambda a: _compile(a[0], a[1], extra, a[2]), jobs))
    LIB_OUT = out_lib
    tmp = LIB_OUT + ".tmp%d" % os.getpid()
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), res.stderr))
    os.replace(tmp, LIB_OUT)
    return LIB_OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
