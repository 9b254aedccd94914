"""Import the pure-Python/Numba reference (LacmoPy) with Numba stubbed out.

Test infrastructure only: used by ``make_golden.py`` in a container that has the
reference sources.  Numba is replaced by identity decorators so the reference
arithmetic runs unchanged as plain Python/NumPy; matplotlib and the plotting
module are replaced by inert modules because only plotting code uses them.

NumPy's AVX-512 (SVML) dispatch must be disabled before NumPy is imported
(``NPY_DISABLE_CPU_FEATURES``) so that NumPy array ``power``/``log``/``exp``
resolve to the scalar glibc libm routines, which is what Numba-compiled code
calls.  ``make_golden.py`` sets it before importing anything.
"""
import os
import sys
import types

import numpy as np


class _Inert(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Inert(name)

    def __call__(self, *a, **k):
        return _Inert("call")


def _numba_stub():
    nb = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    def vectorize(*args, **kwargs):
        def deco(f):
            vf = np.vectorize(f, otypes=[np.float64])

            def wrapper(*a):
                if any(isinstance(x, np.ndarray) and x.ndim > 0 for x in a):
                    return vf(*a)
                return f(*a)
            wrapper.__name__ = f.__name__
            return wrapper
        if len(args) == 1 and callable(args[0]):
            return deco(args[0])
        return deco

    nb.njit = njit
    nb.jit = njit
    nb.vectorize = vectorize
    nb.prange = range
    return nb


def import_reference(ref_root):
    """Put stubs in ``sys.modules`` and import the reference modules.

    Returns a namespace with the reference modules used on the hot path.  The
    working directory is switched to ``ref_root`` because the reference loads
    its collision-efficiency tables by relative path at import time.
    """
    sys.modules["numba"] = _numba_stub()
    for name in ["matplotlib", "matplotlib.pyplot", "matplotlib.ticker",
                 "matplotlib.colors", "mpl_toolkits", "mpl_toolkits.mplot3d",
                 "mpl_toolkits.axes_grid1", "plotting"]:
        sys.modules[name] = _Inert(name)
    sys.path.insert(0, ref_root)
    os.chdir(ref_root)
    import constants, algebra, material_properties, atmosphere, microphysics  # noqa
    import grid, integration, golovin  # noqa
    import collision.all_or_nothing as aon
    import collision.kernel as ker
    import file_handling, generation_SIP_ensemble  # noqa
    ns = types.SimpleNamespace(
        c=constants, alg=algebra, mat=material_properties, atm=atmosphere,
        mp=microphysics, grid=grid, integ=integration, golovin=golovin,
        aon=aon, ker=ker, fh=file_handling, gen=generation_SIP_ensemble)
    return ns
