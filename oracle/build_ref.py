"""Build recipe for the reference orbkit's grid extensions (test infrastructure).

This is part of the oracle, not of the product.  It compiles the reference's own
Cython/C sources for the grid hot path -- exactly the extensions that the
reference's setup.py declares at setup.py:51-75:

  orbkit.cy_grid    <- orbkit/cy_grid.pyx
  orbkit.cy_core    <- orbkit/cy_core.pyx + orbkit/c_grid-based.c + orbkit/c_support.c
  orbkit.cy_overlap <- orbkit/cy_overlap.pyx + orbkit/c_non-grid-based.c + orbkit/c_support.c

and the two detCI extensions (setup.py:76-95) whose grid loops the CI density and
flux-density fixtures come from:

  orbkit.detci.cy_ci        <- orbkit/detci/cy_ci.pyx
  orbkit.detci.cy_occ_check <- orbkit/detci/cy_occ_check.pyx

The sources are read where they lie (the read-only reference tree); every output
(Cython-generated C, objects, the extension modules) goes under ``oracle/_ref/``,
which is git-ignored.  Nothing is copied into the repository.  The reference
tree only exists in the development container, so this recipe is a no-op when it
is absent (the GPU host uses the oracle's own C restatement, ``oracle/okref.c``).

Usage:  python oracle/build_ref.py [REFERENCE_ROOT]
"""
import os
import sys
import sysconfig
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference tree: $ORBKIT_REFERENCE_ROOT, else a checkout named "reference"
# beside this repository
DEFAULT_REF = os.environ.get("ORBKIT_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")

# (module name, [pyx], [extra C sources]) -- mirrors setup.py:51-75 of the reference
EXTENSIONS = [
    ("cy_grid", ["orbkit/cy_grid.pyx"], []),
    ("cy_core", ["orbkit/cy_core.pyx"], ["orbkit/c_grid-based.c", "orbkit/c_support.c"]),
    ("cy_overlap", ["orbkit/cy_overlap.pyx"], ["orbkit/c_non-grid-based.c", "orbkit/c_support.c"]),
    ("detci.cy_ci", ["orbkit/detci/cy_ci.pyx"], []),
    ("detci.cy_occ_check", ["orbkit/detci/cy_occ_check.pyx"], []),
]


def ext_suffix():
    return sysconfig.get_config_var("EXT_SUFFIX") or ".so"


def built_modules(out=OUT):
    """Paths of the built extension modules, or None when not built."""
    paths = {}
    for name, _, _ in EXTENSIONS:
        p = os.path.join(out, "orbkit", *name.split(".")[:-1], name.split(".")[-1] + ext_suffix())
        if not os.path.exists(p):
            return None
        paths[name] = p
    return paths


def build(ref_root=DEFAULT_REF, out=OUT, quiet=True):
    """Cythonize and compile the three extensions; returns {name: path} or None."""
    if not os.path.isdir(os.path.join(ref_root, "orbkit")):
        return None
    try:
        from Cython.Build import cythonize  # noqa: F401  (Cython is container-only)
        from Cython.Compiler import Main as cymain
    except ImportError:
        return None
    import numpy

    cdir = os.path.join(out, "cython")
    odir = os.path.join(out, "obj")
    mdir = os.path.join(out, "orbkit")
    for d in (cdir, odir, mdir):
        os.makedirs(d, exist_ok=True)
    incs = [numpy.get_include(), sysconfig.get_paths()["include"], os.path.join(ref_root, "orbkit")]
    cflags = ["-O2", "-fPIC", "-w"] + ["-I" + i for i in incs]
    for name, pyx, csrc in EXTENSIONS:
        target = os.path.join(mdir, *name.split(".")[:-1], name.split(".")[-1] + ext_suffix())
        os.makedirs(os.path.dirname(target), exist_ok=True)
        srcs = [os.path.join(ref_root, p) for p in pyx + csrc]
        if os.path.exists(target) and all(os.path.getmtime(target) >= os.path.getmtime(s) for s in srcs):
            continue
        cfile = os.path.join(cdir, name + ".c")
        opts = cymain.CompilationOptions(cymain.default_options)
        opts.output_file = cfile
        opts.language_level = 3
        res = cymain.compile(os.path.join(ref_root, pyx[0]), opts, full_module_name="orbkit." + name)
        if res.num_errors:
            raise RuntimeError("cython failed for " + name)
        objs = []
        for src in [cfile] + [os.path.join(ref_root, c) for c in csrc]:
            obj = os.path.join(odir, name + "__" + os.path.basename(src).replace(".c", ".o"))
            subprocess.check_call(["gcc", "-c", src, "-o", obj] + cflags)
            objs.append(obj)
        subprocess.check_call(["gcc", "-shared", "-o", target] + objs + ["-lm"])
        if not quiet:
            print("built", target)
    return built_modules(out)


if __name__ == "__main__":
    r = build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF, quiet=False)
    print(r if r else "reference tree or Cython not available; nothing built")
