"""curadon_gb300 -- curadon's X-ray CT projection operators on GB300 (sm_103a).

Drop-in for the reference package ``curadon``: ``FanGeometry``,
``ConeGeometry``, ``forward(volume, sinogram, geom)``,
``backward(sinogram, volume, geom)``, ``TorchForward``,
``TorchBackprojection`` and the native module's ``plan_2d``, ``forward_2d``,
``backward_2d``, ``forward_3d``, ``backward_3d`` and its stream / event
pools (``stream_pool``, ``get_next_stream``, ...).  The operators are
hand-written CUDA kernels behind the C ABI of ``include/curadon_gb300.h``;
there is no CPU fallback.
"""
from . import backend
from .backend import (adjoint_2d, backward_2d, backward_3d, forward_2d, forward_3d, plan_2d,
                      plan_2d_vec, plan_3d)
from .geometry import ConeGeometry, FanGeometry, FanVecGeometry, geom_to_str
from .ops import TorchBackprojection, TorchForward, adjoint, backward, forward
from .pools import (event, event_pool, event_view, get_event, get_next_event, get_next_stream,
                     get_stream, stream, stream_pool, stream_view)

__all__ = [
    "FanGeometry", "FanVecGeometry", "ConeGeometry", "geom_to_str", "forward", "backward",
    "adjoint", "TorchForward", "TorchBackprojection", "plan_2d", "plan_2d_vec", "plan_3d",
    "forward_2d", "backward_2d", "forward_3d", "backward_3d", "backend",
    "event", "event_view", "event_pool", "stream", "stream_view", "stream_pool",
    "get_next_stream", "get_stream", "get_next_event", "get_event",
]
__version__ = "1.0.0"
