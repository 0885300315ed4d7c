"""GB300 finite-element assembly engine for FEDDLib's element-loop hot path.

The compute path is the in-tree CUDA library libfeddgpu.so (built by
feddlib_gb300.build); this package only binds it.
"""
from ._capi import (ANISO_FIBER, JACOBIAN, LAPLACE, LINEAR_ELASTICITY, NAVIER_STOKES,  # noqa: F401
                    NONLINEAR_ELASTICITY, NONLINEAR_ELASTICITY2, RESIDUAL, FeddError, lib)
from .fe import (FE, Assembler, CsrMatrix, Trainer, detF_scaled_field, fourier_field, medit_read,  # noqa: F401
                 medit_write, p2_of_p1, structured_mesh, structured_mesh_device, uniform_field)

__all__ = ["FE", "Assembler", "CsrMatrix", "Trainer", "structured_mesh", "fourier_field", "uniform_field",
           "structured_mesh_device", "detF_scaled_field", "p2_of_p1", "medit_read", "medit_write",
           "FeddError", "lib"]
