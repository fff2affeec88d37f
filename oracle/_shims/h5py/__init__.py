"""Import stub of h5py for tests that import pyflowreg's motion_correction
package (its I/O modules import h5py at module top).  The tests pass arrays,
never files, so every attribute access fails loudly."""


def __getattr__(name):
    raise ImportError(f"h5py is not installed here (test stub); h5py.{name} is unavailable")
