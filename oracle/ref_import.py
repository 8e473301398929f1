"""Import the reference batoid package (test infrastructure, oracle only).

The reference's Python package is imported from its own source tree, and its
compiled ``_batoid`` module from ``oracle/_ref`` (built by ``oracle/Makefile.ref``
from the reference's sources).  GalSim, matplotlib and PyYAML are not installed
here; the trace, wavefront and Huygens paths never call them, so minimal stub
modules that define only the imported names are registered first.  Nothing in
the product imports this module: it exists to generate and check golden
vectors in this container.
"""
import importlib.util
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BUILD = os.path.join(HERE, "_ref")


def _stub(name, **attrs):
    mod = types.ModuleType(name)
    mod.__dict__.update(attrs)
    sys.modules[name] = mod
    return mod


def _install_stubs():
    if "galsim" not in sys.modules:
        def _missing(*args, **kwargs):
            raise RuntimeError("galsim is not installed (stub)")
        zern = _stub("galsim.zernike", Zernike=_missing, zernikeBasis=_missing,
                     zernikeGradBases=_missing)
        _stub("galsim", zernike=zern).__path__ = []
    if "matplotlib" not in sys.modules:
        mpl = _stub("matplotlib")
        mpl.__path__ = []  # mark as a package so submodule imports resolve
        mpl.pyplot = _stub("matplotlib.pyplot")
        mpl.figure = _stub("matplotlib.figure", Figure=object)
        mpl.gridspec = _stub("matplotlib.gridspec", GridSpec=object)
        _stub("mpl_toolkits").__path__ = []
        _stub("mpl_toolkits.mplot3d", Axes3D=object)
        _stub("mpl_toolkits.axes_grid1", make_axes_locatable=lambda *a, **k: None)


def import_reference(ref_root=None):
    """Return the reference ``batoid`` module, or raise ImportError."""
    if "batoid" in sys.modules and getattr(sys.modules["batoid"], "_is_ref", False):
        return sys.modules["batoid"]
    ref_root = ref_root or os.environ.get("BATOID_REF")
    if not ref_root:
        raise ImportError("reference root not given: pass it or set BATOID_REF")
    pkg = os.path.join(ref_root, "batoid")
    if not os.path.isdir(pkg):
        raise ImportError(f"reference sources not found at {pkg}")
    if not any(f.startswith("_batoid") and f.endswith(".so") for f in os.listdir(REF_BUILD)
               if os.path.isdir(REF_BUILD)):
        raise ImportError("oracle/_ref/_batoid*.so missing: run make -f oracle/Makefile.ref")
    _install_stubs()
    # _version.py is generated by the reference's setup.py; provide it.
    if "batoid._version" not in sys.modules:
        _stub("batoid._version", __version__="ref")
    spec = importlib.util.spec_from_file_location(
        "batoid", os.path.join(pkg, "__init__.py"),
        submodule_search_locations=[pkg, REF_BUILD])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["batoid"] = mod
    try:
        spec.loader.exec_module(mod)
    except Exception:
        del sys.modules["batoid"]
        raise
    mod._is_ref = True
    return mod
