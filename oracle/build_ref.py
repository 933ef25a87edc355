"""Build recipe for the reference's only compiled piece, the ``Domain`` extension.

Test infrastructure: the output is used only to run the unmodified reference
(a pure-Python package plus this one Cython/C extension) in the build
container, to generate and check the golden fixtures under ``tests/golden/``.

The reference compiles ``micmec/pes/ext.pyx`` together with ``domain.c``
(reference setup.py:7-12). This recipe runs Cython and gcc on those two
source files where they lie, and writes everything into ``oracle/_ref/``
(git-ignored), never into the read-only reference tree.
"""

import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("MICMEC_REFERENCE", "/root/reference")


def ext_path():
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    return os.path.join(OUT, "micmec_ref_ext" + suffix)


def build(force=False):
    """Compile the reference ``Domain`` extension; return the path of the .so."""
    target = ext_path()
    if os.path.exists(target) and not force:
        return target
    import numpy

    pes = os.path.join(REF, "micmec", "pes")
    os.makedirs(os.path.join(OUT, "build"), exist_ok=True)
    c_file = os.path.join(OUT, "build", "ext.c")
    subprocess.check_call(
        [sys.executable, "-m", "cython", "-3", "--module-name", "micmec.pes.ext",
         "-I", pes, os.path.join(pes, "ext.pyx"), "-o", c_file]
    )
    cmd = [
        "gcc", "-shared", "-fPIC", "-O2",
        "-I", sysconfig.get_paths()["include"], "-I", numpy.get_include(), "-I", pes,
        c_file, os.path.join(pes, "domain.c"), "-o", target,
    ]
    subprocess.check_call(cmd)
    return target


def import_reference():
    """Import the reference ``micmec`` package with the compiled ``Domain`` in place.

    Needs the molmod/h5py stand-ins under ``tests/golden/standin`` on ``sys.path``.
    """
    import importlib.machinery
    import importlib.util

    so = build()
    standin = os.path.join(os.path.dirname(HERE), "tests", "golden", "standin")
    for p in (standin, REF, os.path.dirname(HERE)):
        if p not in sys.path:
            sys.path.insert(0, p)
    loader = importlib.machinery.ExtensionFileLoader("micmec.pes.ext", so)
    spec = importlib.util.spec_from_file_location("micmec.pes.ext", so, loader=loader)
    import micmec.pes  # noqa: F401  (the package itself is pure Python)

    mod = importlib.util.module_from_spec(spec)
    sys.modules["micmec.pes.ext"] = mod
    loader.exec_module(mod)
    import micmec

    return micmec


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
