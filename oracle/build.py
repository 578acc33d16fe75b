"""Build recipe for the oracle (test infrastructure only).

1. ``liboracle.so``: the plain-C restatement (joker_oracle.c + kepler.c),
   compiled with gcc into ``oracle/_build/``.
2. ``oracle/_ref``: the reference's own, unmodified Cython likelihood
   (thejoker/src/fast_likelihood.pyx) compiled from where it lies in the
   reference checkout.  Cython runs only where the reference and Cython are
   present; it writes ``oracle/_ref/fast_likelihood.c``.  Wherever that
   generated C file exists (it travels with the repository copy), gcc turns it
   into ``oracle/_ref/fast_likelihood<EXT_SUFFIX>``, linked against
   ``kepler.c`` in place of the absent twobody C library.
"""
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# the reference checkout: JOKER_REFERENCE_ROOT, else where this container mounts it
REFERENCE_ROOT = os.environ.get("JOKER_REFERENCE_ROOT", "/root/reference")
REF_PYX = os.path.join(REFERENCE_ROOT, "thejoker", "src", "fast_likelihood.pyx")
ORACLE_SO = os.path.join(BUILD, "liboracle.so")


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("joker_oracle.c", "kepler.c")]
    if force or _newer(ORACLE_SO, srcs + [os.path.join(HERE, "kepler.h")]):
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-o", ORACLE_SO] + srcs + ["-lm"]
        subprocess.run(cmd, check=True)
    return ORACLE_SO


def ref_so_path():
    return os.path.join(REF_OUT, "fast_likelihood" + sysconfig.get_config_var("EXT_SUFFIX"))


def cythonize_reference():
    """Translate the reference .pyx to C (needs the reference checkout and Cython)."""
    if not os.path.exists(REF_PYX):
        return None
    try:
        import Cython  # noqa: F401
    except ImportError:
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    out_c = os.path.join(REF_OUT, "fast_likelihood.c")
    if _newer(out_c, [REF_PYX]):
        cmd = [sys.executable, "-m", "cython", "-3", "--module-name",
               "thejoker.src.fast_likelihood", REF_PYX, "-o", out_c]
        subprocess.run(cmd, check=True, capture_output=True)
    return out_c


def build_reference(force=False):
    """Compile the reference Cython module; returns the .so path or None."""
    cythonize_reference()
    out_c = os.path.join(REF_OUT, "fast_likelihood.c")
    if not os.path.exists(out_c):
        return None
    import numpy as np
    so = ref_so_path()
    deps = [out_c, os.path.join(HERE, "kepler.c"), os.path.join(HERE, "kepler.h")]
    if force or _newer(so, deps):
        inc = sysconfig.get_paths()["include"]
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-w",
               "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
               "-I", inc, "-I", np.get_include(), "-I", os.path.join(HERE, "ref_shim"),
               out_c, os.path.join(HERE, "kepler.c"), "-o", so, "-lm"]
        subprocess.run(cmd, check=True)
    return so


def build_all():
    build_oracle()
    try:
        return build_reference()
    except (subprocess.CalledProcessError, OSError) as exc:  # reported, not fatal
        print(f"oracle: reference Cython module not built: {exc}", file=sys.stderr)
        return None


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
