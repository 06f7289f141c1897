"""Build recipe for the *reference* raypier Cython tracer, used only as a test oracle.

This is test infrastructure: it compiles the reference implementation of the
non-sequential tracing hot path (``raypier/core/{ctracer,cmaterials,cfaces,cshapes,
cdistortions}.pyx``) and of the E-field summation that consumes its output
(``cfields.pyx``) so that tests, golden-vector generation and the CPU
baseline in ``bench.py`` can run the reference's own code.  Nothing in the
product package imports it.

Two stages, both writing only under ``oracle/_ref/`` (git-ignored):

1. ``cythonize`` (needs Cython and the reference sources): copies the six
   Cython modules plus ``ctracer.pxd`` and ``core/{tracer,fields,utils}.py``
   from the reference checkout into ``oracle/_ref/raypier/core/`` and generates the
   ``.c`` files next to them.  Runs in the development container.
2. ``compile`` (needs only gcc, Python headers and numpy headers): compiles each
   generated ``.c`` into an extension module with ``-O2 -ffp-contract=off``
   (no ``-march=native``: FMA contraction would change float results) and
   ``-fopenmp`` (``cdistortions`` and ``cfields`` call the OpenMP runtime).  Runs on any host
   the generated C travelled to, including an aarch64 host.

``load()`` imports the compiled modules through a stub ``raypier`` package,
because the real ``raypier/__init__.py`` imports traits/VTK, which are absent.
"""
from __future__ import annotations

import importlib
import os
import shutil
import subprocess
import sys
import sysconfig
import types
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
PKG_DIR = os.path.join(REF_OUT, "raypier", "core")
MODULES = ["ctracer", "cmaterials", "cfaces", "cshapes", "cdistortions", "cfields"]
# pure-Python modules of the reference imported next to them
PY_MODULES = ["tracer", "fields", "utils"]
# The reference checkout: RP_REFERENCE_SRC, else a directory named `reference`
# beside this repository's root (the layout the build scripts are run in).
DEFAULT_SRC = os.environ.get("RP_REFERENCE_SRC") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def _ext_suffix() -> str:
    return sysconfig.get_config_var("EXT_SUFFIX") or ".so"


def cythonize(src_root: str = DEFAULT_SRC) -> None:
    """Stage 1: copy the reference hot-path sources and generate C with Cython."""
    core = os.path.join(src_root, "raypier", "core")
    if not os.path.isdir(core):
        raise FileNotFoundError(f"reference sources not found at {core}")
    os.makedirs(PKG_DIR, exist_ok=True)
    for name in [m + ".pyx" for m in MODULES] + ["ctracer.pxd"] + [m + ".py" for m in PY_MODULES]:
        shutil.copyfile(os.path.join(core, name), os.path.join(PKG_DIR, name))
    for init in (os.path.join(REF_OUT, "raypier", "__init__.py"),
                 os.path.join(PKG_DIR, "__init__.py")):
        open(init, "w").close()
    import numpy
    from Cython.Build import cythonize as _cy
    cwd = os.getcwd()
    os.chdir(REF_OUT)
    try:
        _cy([os.path.join("raypier", "core", m + ".pyx") for m in MODULES],
            include_path=[numpy.get_include(), REF_OUT], language_level="3",
            quiet=True, nthreads=len(MODULES))
    finally:
        os.chdir(cwd)


def have_generated_c() -> bool:
    return all(os.path.exists(os.path.join(PKG_DIR, m + ".c")) for m in MODULES)


def have_built() -> bool:
    suf = _ext_suffix()
    return all(os.path.exists(os.path.join(PKG_DIR, m + suf)) for m in MODULES)


def _compile_one(mod: str) -> None:
    import numpy
    src = os.path.join(PKG_DIR, mod + ".c")
    out = os.path.join(PKG_DIR, mod + _ext_suffix())
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return
    inc = sysconfig.get_paths()["include"]
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-strict-aliasing", "-fPIC",
           "-shared", "-fopenmp", "-w",
           "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
           "-I", inc, "-I", numpy.get_include(), src, "-o", out + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)


def compile_generated() -> None:
    """Stage 2: compile the generated C (in parallel) into extension modules."""
    if not have_generated_c():
        raise FileNotFoundError("generated reference C is missing; run cythonize() first")
    with ThreadPoolExecutor(len(MODULES)) as ex:
        list(ex.map(_compile_one, MODULES))


def build(src_root: str = DEFAULT_SRC) -> bool:
    """Build what can be built here.  Returns True when the reference modules exist."""
    if not have_generated_c():
        try:
            import Cython  # noqa: F401
        except ImportError:
            return False
        if not os.path.isdir(os.path.join(src_root, "raypier", "core")):
            return False
        cythonize(src_root)
    compile_generated()
    return have_built()


def load():
    """Import the compiled reference modules through a stub ``raypier`` package.

    Returns a namespace with ``ctracer, cmaterials, cfaces, cshapes,
    cdistortions, cfields, tracer, fields, utils``.
    """
    if not have_built():
        raise ImportError("reference tracer is not built (oracle/build_ref.py)")
    if "raypier" not in sys.modules or not getattr(sys.modules["raypier"], "_rp_stub", False):
        pkg = types.ModuleType("raypier")
        pkg.__path__ = [os.path.join(REF_OUT, "raypier")]
        pkg._rp_stub = True
        sys.modules["raypier"] = pkg
        for k in [k for k in sys.modules if k.startswith("raypier.")]:
            del sys.modules[k]
    ns = types.SimpleNamespace()
    for m in MODULES + PY_MODULES:
        setattr(ns, m, importlib.import_module("raypier.core." + m))
    return ns


if __name__ == "__main__":
    ok = build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_SRC)
    print("reference built" if ok else "reference not buildable here")
