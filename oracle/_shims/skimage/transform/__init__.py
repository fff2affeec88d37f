"""Stub of ``skimage.transform.resize``; off the optical-flow path."""


def resize(*args, **kwargs):
    raise NotImplementedError(
        "skimage.transform.resize is not available in the oracle shim "
        "(it is not used by get_displacement)"
    )
