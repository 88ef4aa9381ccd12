"""Recipe: the reference viewer's own GPU evaluator, built as a checker.

Test infrastructure only; nothing under ``scwatter_gb300/`` uses it.

``gpuEvaluator.cu`` (gpuEvaluator.cu:1-165) needs only thrust, the CUDA runtime, tira's
``HANDLE_ERROR`` macro and the unpacked-wave globals of ``cpuEvaluator.h``, so it compiles on
its own.  ``fetch()`` copies ``gpuEvaluator.cu`` and ``gpuEvaluator.h`` UNCHANGED from the
reference checkout into the git-ignored ``oracle/_ref/src/`` (when the checkout is present; the
copy travels with the working tree to the GPU machine, which has no checkout), and records
their SHA-256.  ``build()`` compiles, for sm_103a:

* ``oracle/_ref/libref_gpu_evaluator.so``: the reference's kernels behind
  ``oracle/ref_harness.cu`` (the globals and a C entry ``scwref_evaluate``), with the stand-in
  headers of ``oracle/ref_stubs/`` in place of tira and of the Eigen / FFTW / MKL / glm
  includes that cpuEvaluator.h pulls in;
* ``oracle/_ref/libref_shim.so``: the same harness over the drop-in shim
  ``scwatter_gb300/shim/gpuEvaluator_gb300.cu`` compiled against the reference's own
  ``gpuEvaluator.h``, linked to ``libscwatter_gb300.so``.

Nothing here runs the reference's build system (it needs cmake, tira, Eigen, FFTW, MKL, Boost,
glm and the GL stack, none of which is present).
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF = os.environ.get("SCW_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
STUBS = os.path.join(HERE, "ref_stubs")
FILES = ("gpuEvaluator.cu", "gpuEvaluator.h")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_REF = os.path.join(OUT, "libref_gpu_evaluator.so")
LIB_SHIM = os.path.join(OUT, "libref_shim.so")


def _sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def fetch() -> bool:
    """Copies the two reference files unchanged; False when no reference checkout is present."""
    if not all(os.path.isfile(os.path.join(REF, f)) for f in FILES):
        return False
    os.makedirs(SRC, exist_ok=True)
    digests = {}
    for f in FILES:
        src, dst = os.path.join(REF, f), os.path.join(SRC, f)
        if not os.path.exists(dst) or _sha(dst) != _sha(src):
            shutil.copyfile(src, dst)
        digests[f] = _sha(dst)
    json.dump(digests, open(os.path.join(SRC, "SHA256.json"), "w"), indent=1)
    return True


def sources_present() -> bool:
    return all(os.path.isfile(os.path.join(SRC, f)) for f in FILES)


def _nvcc(out, srcs, extra=()):
    deps = list(srcs) + [os.path.join(HERE, "ref_harness.cu")]
    for d in (STUBS, os.path.join(ROOT, "include")):
        for dirpath, _, names in os.walk(d):
            deps += [os.path.join(dirpath, n) for n in names if n.endswith(".h")]
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(p) for p in deps if os.path.exists(p)):
        return
    cmd = [NVCC, *ARCH, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-I", SRC, "-I", STUBS,
           "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "ref_harness.cu"), *srcs, "-o", out, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference checker build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build() -> bool:
    """Builds both checker libraries; False when the reference sources are not available."""
    fetch()
    if not sources_present():
        return False
    import concurrent.futures as cf
    lib_dir = os.path.join(ROOT, "scwatter_gb300")
    jobs = [(LIB_REF, [os.path.join(SRC, "gpuEvaluator.cu")], []),
            (LIB_SHIM, [os.path.join(ROOT, "scwatter_gb300", "shim", "gpuEvaluator_gb300.cu")],
             ["-L", lib_dir, "-lscwatter_gb300", "-Xlinker", "-rpath=$ORIGIN/../../scwatter_gb300"])]
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        for f in [ex.submit(_nvcc, *j) for j in jobs]:
            f.result()
    return True


if __name__ == "__main__":
    print(build())
