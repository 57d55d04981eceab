"""Loads the reference's own Python wrappers (Corrfunc/*.py, staged unchanged into
oracle/_ref/src/py by oracle/build_ref.py) on top of this project's CPython extension modules.

The wrappers import two third-party packages that are not installed here and matter only for
Python 2 and notebooks: ``future.utils.bytes_to_native_str`` (bytes -> str on Python 3) and
``wurlitzer.pipes`` (redirects C-level stdout/stderr into notebook cells).  Minimal stand-ins
are installed for them; ``Corrfunc._countpairs`` and ``Corrfunc._countpairs_mocks`` are the
modules ``corrfunc_gb300._countpairs`` and ``corrfunc_gb300._countpairs_mocks``.
"""
import contextlib
import os
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PY_DIR = os.path.join(ROOT, "oracle", "_ref", "src", "py")


def _install_stand_ins():
    if "future.utils" not in sys.modules:
        future = types.ModuleType("future")
        utils = types.ModuleType("future.utils")
        utils.bytes_to_native_str = lambda b, encoding="utf-8": b.decode(encoding)
        future.utils = utils
        sys.modules["future"] = future
        sys.modules["future.utils"] = utils
    if "wurlitzer" not in sys.modules:
        wz = types.ModuleType("wurlitzer")

        @contextlib.contextmanager
        def pipes(stdout=None, stderr=None, **kw):
            yield stdout, stderr

        wz.pipes = pipes
        sys.modules["wurlitzer"] = wz


def load():
    """The reference's Corrfunc package running on corrfunc_gb300's extension modules (skips the
    calling test when the wrappers are not staged or the modules are not built)."""
    if not os.path.isdir(os.path.join(PY_DIR, "Corrfunc")):
        pytest.skip("reference Python wrappers not staged in oracle/_ref/src/py")
    import corrfunc_gb300
    try:
        import corrfunc_gb300._countpairs as cp
        import corrfunc_gb300._countpairs_mocks as cpm
    except ImportError as exc:
        pytest.skip("CPython extension modules not built: %s" % exc)
    _install_stand_ins()
    if PY_DIR not in sys.path:
        sys.path.insert(0, PY_DIR)
    sys.modules["Corrfunc._countpairs"] = cp
    sys.modules["Corrfunc._countpairs_mocks"] = cpm
    import Corrfunc
    assert os.path.dirname(os.path.dirname(Corrfunc.__file__)) == PY_DIR, Corrfunc.__file__
    Corrfunc._countpairs = cp
    Corrfunc._countpairs_mocks = cpm
    corrfunc_gb300.library()
    return Corrfunc
