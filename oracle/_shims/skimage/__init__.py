"""Test-infrastructure shim for ``skimage`` (absent in this image).

pyflowreg imports ``skimage.transform.resize`` at module top in
``util/resize_util.py:4`` but uses it only in ``resize_image_skimage``, which
is not on the optical-flow path.  The stub raises if it is ever called.
"""
