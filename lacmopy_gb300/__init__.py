"""lacmopy_gb300: GB300 (sm_103a) CUDA implementation of LacmoPy's per-timestep
super-droplet hot path (advection + re-index, Newton condensation with grid
feedback, all-or-nothing collisions), behind a C ABI (include/lacmo_gb300.h).

Modules mirror the reference's step functions by name and argument list:
``integration`` (integration.py / grid.py / microphysics.py helpers) and
``collision`` (collision/all_or_nothing.py, collision/box_model.py driver).
``DeviceState`` keeps a state resident on the GPU between steps.
"""
__all__ = ["BatchState", "DeviceState"]


def __getattr__(name):
    # the device classes import torch; the pure-NumPy modules (synthetic,
    # tables, constants) stay importable without it
    if name in __all__:
        from . import device
        return getattr(device, name)
    raise AttributeError(name)
