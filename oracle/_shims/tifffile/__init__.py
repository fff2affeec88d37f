"""Import stub of tifffile for tests that import pyflowreg's motion_correction
package (its I/O modules import tifffile at module top).  The tests pass
arrays, never files, so every attribute access fails loudly."""


def __getattr__(name):
    raise ImportError(f"tifffile is not installed here (test stub); tifffile.{name} is unavailable")
