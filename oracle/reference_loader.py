"""Import the reference package (``skfemntv``) from its checkout, with the
``_skfn`` extension compiled by ``oracle/build_ref.sh`` into ``oracle/_ref``.

Test infrastructure only: used to pin the CPU oracle and to regenerate the
golden fixtures under ``tests/golden``.  Nothing is copied out of the
reference checkout; its Python sources are imported in place.
"""
from __future__ import annotations

import glob
import importlib.machinery
import importlib.util
import os
import sys

REFERENCE_ROOT = os.environ.get("SKFEM_REFERENCE", "/root/reference")
_HERE = os.path.dirname(os.path.abspath(__file__))


def available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "python", "skfemntv")) and bool(
        glob.glob(os.path.join(_HERE, "_ref", "_skfn*.so"))
    )


def load():
    """Return the reference ``skfemntv`` module (raises if unavailable)."""
    if "skfemntv" in sys.modules:
        return sys.modules["skfemntv"]
    so = glob.glob(os.path.join(_HERE, "_ref", "_skfn*.so"))
    if not so:
        raise ImportError("reference extension not built; run oracle/build_ref.sh")
    pkg_dir = os.path.join(REFERENCE_ROOT, "python", "skfemntv")
    loader = importlib.machinery.ExtensionFileLoader("skfemntv._skfn", so[0])
    spec = importlib.util.spec_from_file_location("skfemntv._skfn", so[0], loader=loader)
    ext = importlib.util.module_from_spec(spec)
    loader.exec_module(ext)
    sys.modules["skfemntv._skfn"] = ext
    pspec = importlib.util.spec_from_file_location(
        "skfemntv", os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir]
    )
    pkg = importlib.util.module_from_spec(pspec)
    sys.modules["skfemntv"] = pkg
    pspec.loader.exec_module(pkg)
    return pkg
