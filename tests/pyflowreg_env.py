"""Imports pyflowreg, the unmodified reference package, for the tests of the
drop-in boundary.  It is looked up as an installed package, in
``baseline/_ref`` (where ``pip install --target baseline/_ref <pyflowreg
checkout>`` puts it) or under the directory in $PYFLOWREG_SRC; the test
skips when none has it.  Modules pyflowreg imports that are absent here
(numba, cv2, skimage, tifffile, h5py, hdf5storage) come from the test shims
in oracle/_shims, appended to sys.path so that installed ones take precedence.
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIMS = os.path.join(REPO, "oracle", "_shims")


def import_pyflowreg():
    if SHIMS not in sys.path:
        sys.path.append(SHIMS)
    try:
        import pyflowreg  # noqa: F401

        return pyflowreg
    except ImportError:
        pass
    for cand in (os.path.join(REPO, "baseline", "_ref"), os.environ.get("PYFLOWREG_SRC")):
        if cand and os.path.isdir(os.path.join(cand, "pyflowreg")):
            sys.path.insert(0, cand)
            break
    else:
        pytest.skip("pyflowreg is not importable (install it into baseline/_ref or set PYFLOWREG_SRC)")
    try:
        import pyflowreg

        return pyflowreg
    except ImportError as e:
        pytest.skip(f"pyflowreg does not import here: {e}")


def import_motion_correction():
    """pyflowreg.motion_correction needs pydantic (OFOptions); skip without it."""
    pytest.importorskip("pydantic")
    import_pyflowreg()
    import pyflowreg.motion_correction as mc

    return mc
