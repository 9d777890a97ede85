"""sfbgpu - GB300 implementation of SuperFaB's catalogue -> SFB coefficient path.

Host-side mirror of the reference API for this path (``AnlmModes``,
``ConfigurationSpaceModes``, ``cat2amln``, ``field2anlm``, ``anlm2field``,
``win_rhat_ln``, ...).  The transforms run in ``libsfbgpu.so`` (hand-written
CUDA for sm_103a) behind the C ABI declared in ``include/sfb_gpu.h``.
Mode setup (k_nl roots, splines) is host code, as it is on the Julia side.
"""

from .modes import (AnlmModes, ClnnModes, estimate_nside, getidx, getidx0, getidx_lnn, getlmsize, getlnn,
                    getlnnsize, getnlm, getnlmsize, isvalidnlm)
from .windows import (ConfigurationSpaceModes, SeparableArray, gen_mask, get_rbounds, integrate_window, make_window,
                      window_r)
from .healpix import nside2npix, npix2nside, pix2ang_ring


def xyz2rtp(xyz):
    """Cartesian (3, N) -> (r, theta, phi) (reference src/SphericalFourierBesselDecompositions.jl:517-532)."""
    import numpy as np
    xyz = np.asarray(xyz, float)
    x, y, z = xyz
    r = np.sqrt(x ** 2 + y ** 2 + z ** 2)
    return np.stack([r, np.arccos(z / r), np.arctan2(y / r, x / r)])


def __getattr__(name):
    # GPU entry points load libsfbgpu.so on first use
    import importlib
    if name.startswith("__"):
        raise AttributeError(name)
    _c = importlib.import_module(".cat2anlm", __name__)
    if hasattr(_c, name):
        return getattr(_c, name)
    raise AttributeError(name)
