"""GB300-native channel-flow time step (Fourier-Chebyshev, v-omega_y).

The compute path is the CUDA library ``libchflow.so`` (hand-written sm_103a
kernels behind the C ABI of include/chflow.h).  This package is a thin host
layer over that ABI with the same call sequence as the reference's main loop:

    ch = Channel(cfg)              # set-up   (poiseuilleflow.f90:77-214)
    ch.upload_state(state)         # module arrays (paraandcons.f90:28-38)
    ch.getnonlinear()              # getnonlinear (poiseuilleflow.f90:1380-1612)
    ch.solve()                     # solve loop + (0,0) mode (poiseuilleflow.f90:242-474)
    ch.step(n)                     # n x (getnonlinear + solve)
    state = ch.download_state()

``Batch(cfgs)`` steps an ensemble of independent channels together, and
``restart`` reads and writes the reference's per-rank restart files.
There is no CPU fallback: if the library cannot be loaded, every call raises.
"""
from .config import ChannelConfig, CONFIGS, small  # noqa: F401
from .channel import Batch, Channel, ChannelError, load_library, PRECISION  # noqa: F401
from . import fields, restart  # noqa: F401

__all__ = ["ChannelConfig", "CONFIGS", "small", "Batch", "Channel", "ChannelError", "load_library",
           "PRECISION", "fields", "restart"]
