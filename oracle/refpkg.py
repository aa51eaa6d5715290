"""Import the reference orbkit package in the development container (test infrastructure).

The reference is pure Python on top of three compiled extensions.  This module
loads the extensions built by ``oracle/build_ref.py`` under their package names
(``orbkit.cy_core`` ...), then imports the reference's Python package from the
read-only reference tree.  Harness-only shims make the unmodified reference run
on numpy 2 without its optional plotting/HDF5 dependencies:

  * ``numpy.product``/``numpy.int`` aliases (used at grid.py:75,156 and test/tools.py:9),
  * import-time stubs for h5py / skimage / matplotlib,
  * quiet display (options.quiet / options.no_log).

The reference is never modified.  Only tests and the fixture generator use this;
it returns None when the reference tree is not present (e.g. on the GPU host).
"""
import importlib.util
import os
import sys
import types

# the reference tree: $ORBKIT_REFERENCE_ROOT, else a checkout named "reference"
# beside this repository
REF_ROOT = os.environ.get("ORBKIT_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "reference")


def _stub(name):
    if name in sys.modules:
        return
    try:
        __import__(name)
    except Exception:
        m = types.ModuleType(name)
        m.__path__ = []  # allow submodule imports such as matplotlib.pyplot
        sys.modules[name] = m


def load(build=True):
    """Return the reference ``orbkit`` module, or None if unavailable."""
    if "orbkit" in sys.modules and getattr(sys.modules["orbkit"], "_okg_loaded_from_ref", False):
        return sys.modules["orbkit"]
    if not os.path.isdir(os.path.join(REF_ROOT, "orbkit")):
        return None
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    try:
        import build_ref
    finally:
        sys.path.pop(0)
    mods = build_ref.built_modules()
    if mods is None and build:
        mods = build_ref.build(REF_ROOT)
    if mods is None:
        return None

    import numpy
    if not hasattr(numpy, "product"):
        numpy.product = numpy.prod
    if not hasattr(numpy, "int"):
        numpy.int = int
    for name in ("h5py", "skimage", "skimage.measure", "matplotlib", "matplotlib.pyplot",
                 "mpl_toolkits", "mpl_toolkits.mplot3d"):
        _stub(name)

    for name, path in mods.items():
        full = "orbkit." + name
        if full in sys.modules:
            continue
        spec = importlib.util.spec_from_file_location(full, path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        sys.modules[full] = mod

    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    import orbkit  # noqa: E402  (the reference package)
    orbkit.options.quiet = True
    orbkit.options.no_log = True
    orbkit._okg_loaded_from_ref = True
    return orbkit


def to_reference_qc(ok, qc):
    """The same molecule as the reference's own QCinfo/AOClass/MOClass objects."""
    import numpy
    from orbkit.orbitals import AOClass, MOClass
    from orbkit.qcinfo import QCinfo
    ao = AOClass(seq=[dict(s) for s in qc.ao_spec.data])
    ao.spherical = bool(getattr(qc.ao_spec, "spherical", False))
    ao.update()
    mo = MOClass(seq=[dict(m) for m in qc.mo_spec.data])
    mo.update()
    q = QCinfo()
    q.geo_spec = numpy.array(qc.geo_spec)
    q.geo_info = numpy.array([["X", str(i + 1), "0"] for i in range(len(q.geo_spec))])
    q.ao_spec = ao
    q.mo_spec = mo
    return q
