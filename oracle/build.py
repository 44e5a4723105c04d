"""Build recipe for the CPU oracle (test infrastructure).

* ``build_oracle()`` compiles the C restatement ``oracle/edxr_oracle.c`` into
  ``oracle/_build/libedxr_oracle.so`` with the flags its arithmetic contract
  needs: ``-fwrapv`` (int32 wraparound, as SSE paddd/pmulld) and
  ``-ffp-contract=off`` (no fused multiply-add).
* ``build_ref()`` compiles the reference's own pipeline sources, unmodified and
  where they lie (``EDXRaster/Core/Renderer.cpp``, ``FrameBuffer.cpp``,
  ``Scene.cpp`` and the headers they include), against the project-written
  EDXUtil shim in ``oracle/shim`` plus ``oracle/ref_harness.cpp``, into
  ``oracle/_ref/libedxr_ref.so``.  It needs the reference checkout: ``EDXR_REFERENCE_ROOT``, else a
  ``reference`` directory beside the repository's own; without it the
  reference build is skipped and only the restatement exists.

Run ``python -m oracle.build`` to build both.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libedxr_oracle.so")
REF_SO = os.path.join(REF_DIR, "libedxr_ref.so")

REFERENCE_ROOT = os.environ.get("EDXR_REFERENCE_ROOT",
                                os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
FLAGS = ["-O2", "-fPIC", "-fwrapv", "-ffp-contract=off"]


def _newer(target: str, sources) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, "edxr_oracle.c"), os.path.join(HERE, "edxr_oracle.h")]
    if force or not _newer(ORACLE_SO, srcs):
        tmp = ORACLE_SO + ".tmp%d" % os.getpid()
        _run(["gcc", "-std=c11", *FLAGS, "-shared", "-o", tmp, srcs[0], "-lpthread", "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_ROOT, "EDXRaster", "Core", "Renderer.cpp"))


def build_ref(force: bool = False) -> str | None:
    if not reference_available():
        return None
    core = os.path.join(REFERENCE_ROOT, "EDXRaster", "Core")
    tus = [os.path.join(core, "Renderer.cpp"), os.path.join(core, "FrameBuffer.cpp"),
           os.path.join(core, "Scene.cpp"), os.path.join(HERE, "ref_harness.cpp")]
    shim = os.path.join(HERE, "shim")
    deps = list(tus)
    for root, _, files in os.walk(shim):
        deps += [os.path.join(root, f) for f in files]
    for root, _, files in os.walk(os.path.join(REFERENCE_ROOT, "EDXRaster")):
        deps += [os.path.join(root, f) for f in files if f.endswith(".h")]
    if not force and _newer(REF_SO, deps):
        return REF_SO
    os.makedirs(REF_DIR, exist_ok=True)
    objs = []

    def compile_one(src):
        obj = os.path.join(REF_DIR, os.path.splitext(os.path.basename(src))[0] + ".o")
        # -w: the reference is MSVC-era code and warns heavily under g++;
        # -Wno-narrowing: it brace-initialises uint arrays from int values
        # (Clipper.h:158,176), an error in strict C++11.
        _run(["g++", "-std=c++17", *FLAGS, "-w", "-Wno-narrowing", "-I", shim, "-I", core,
              "-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(max_workers=4) as ex:
        objs = list(ex.map(compile_one, tus))
    tmp = REF_SO + ".tmp%d" % os.getpid()
    _run(["g++", "-shared", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv) or "reference sources not present: reference build skipped")
