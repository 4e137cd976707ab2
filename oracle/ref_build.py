"""Recipe: the reference's own interpolation module, compiled to bytecode in
oracle/_ref/ so that it can run where its sources are absent.

Test and benchmark infrastructure only (the CPU baseline of bench.py); the
package never imports it.  The reference (DurhamDecLab/ARBInterp v1.8) is
one pure-Python/NumPy file, src/ARBInterp/ARBInterp.py; nothing in it is
compiled to machine code, so its "build" is CPython's own byte-compilation
of that file, unmodified, where it lies.  The output,
oracle/_ref/arb_reference.pyc, is git-ignored: it is regenerated by
``build()`` in any container that holds the reference sources and is loaded
with a sourceless loader (``load()``) elsewhere.  The bytecode is tied to the
CPython minor version (3.12 here and on the GPU host).
"""
from __future__ import annotations

import importlib.machinery
import importlib.util
import os
import py_compile
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "arb_reference.pyc")
SRC = os.path.join(os.sep, "root", "reference", "src", "ARBInterp", "ARBInterp.py")


def build(src: str = SRC) -> str | None:
    """Byte-compile the reference module into oracle/_ref/ (None if the
    reference sources are not present)."""
    if not os.path.exists(src):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    if os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(src):
        return OUT
    py_compile.compile(src, cfile=OUT, doraise=True, invalidation_mode=py_compile.PycInvalidationMode.UNCHECKED_HASH)
    return OUT


def available() -> bool:
    return os.path.exists(OUT)


def load():
    """The reference module (tricubic, quadcubic) from the compiled bytecode."""
    if not available():
        raise FileNotFoundError(f"{OUT} is missing: run oracle/ref_build.py where the reference sources are")
    loader = importlib.machinery.SourcelessFileLoader("arb_reference", OUT)
    spec = importlib.util.spec_from_loader("arb_reference", loader)
    mod = importlib.util.module_from_spec(spec)
    loader.exec_module(mod)
    return mod


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else SRC))
