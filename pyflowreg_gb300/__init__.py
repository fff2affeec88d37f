"""GB300 (sm_103a) backend for pyflowreg's variational optical-flow path.

Drop-in replacements for pyflowreg's ``get_displacement``,
``imregister_wrapper`` and the ``level_solver_backend`` seam, computed by
hand-written CUDA kernels behind the C ABI in ``include/flowreg_gb300.h``.
``register()`` adds the ``"flowreg_gb300"`` flow backend and the ``"gb300"``
batch executor to an importable pyflowreg.
"""

from .api import (  # noqa: F401
    Plan,
    clear_plans,
    get_displacement,
    get_displacement_batch,
    get_displacement_device,
    get_motion_tensor_gc,
    get_motion_tensor_gray,
    get_plan,
    imregister_device,
    imregister_wrapper,
    imresize_fused_gauss_cubic,
    level_solver,
    make_params,
    median_filter5,
)
from .backend import register  # noqa: F401

__all__ = [
    "Plan",
    "clear_plans",
    "get_displacement",
    "get_displacement_batch",
    "get_displacement_device",
    "get_motion_tensor_gc",
    "get_motion_tensor_gray",
    "get_plan",
    "imregister_device",
    "imregister_wrapper",
    "imresize_fused_gauss_cubic",
    "level_solver",
    "make_params",
    "median_filter5",
    "register",
]
