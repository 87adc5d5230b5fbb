"""GB300-native SSFM z-march for focused-Gaussian-beam SHG (drop-in for the
fftwf/RK4/Jacobi path of alfredos84/SHG_Focused_Gaussian_Beams).

The compute runs in ``_build/libshg_gb300.so`` (CUDA, sm_103a) behind the C ABI of
``include/shg.h``; ``solver`` is its Python mirror.
"""
from .workloads import (CRYSTAL_QPM50, CRYSTAL_REFERENCE, Crystal, Instance, config_plain_128,  # noqa: F401
                        config_sweep, config_thermal_256, sellmeier_n)

__all__ = ["Solver", "Sweep", "dft2d_device", "Crystal", "Instance", "CRYSTAL_REFERENCE", "CRYSTAL_QPM50"]


def __getattr__(name):
    if name in ("Solver", "Sweep", "dft2d_device"):
        from . import solver
        return getattr(solver, name)
    raise AttributeError(name)
