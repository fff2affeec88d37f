"""Import stub of hdf5storage for tests that import pyflowreg's motion_correction
package (its I/O modules import hdf5storage at module top).  The tests pass arrays,
never files, so every attribute access fails loudly."""


def __getattr__(name):
    raise ImportError(f"hdf5storage is not installed here (test stub); hdf5storage.{name} is unavailable")
