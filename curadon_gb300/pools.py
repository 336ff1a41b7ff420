"""CUDA stream and event pools with the reference's Python surface.

The reference exports from its native module (stream.cu:7-36 over
pool.hpp:16-215): owning ``event`` and ``stream`` objects, non-owning
``event_view`` and ``stream_view`` handles, fixed-size ``event_pool`` /
``stream_pool`` objects that hand out views round-robin
(``get_next_*``) or by index modulo the pool size (``get_*``), and
module-level ``get_next_stream`` / ``get_stream`` / ``get_next_event`` /
``get_event`` over process-wide pools of 16.  The same classes and functions
here wrap PyTorch's CUDA streams and events (plumbing only), so a pool
stream can also carry this package's operators, which run on the current
stream: ``with curadon_gb300.get_next_stream().as_current(): forward(...)``.
``value()`` returns the raw ``cudaStream_t`` / ``cudaEvent_t`` handle as an
integer, as the reference's implicit conversions do.
"""
from __future__ import annotations

import itertools
import threading
from typing import Optional, Union

import torch

__all__ = ["event", "event_view", "event_pool", "stream", "stream_view", "stream_pool",
           "get_next_stream", "get_stream", "get_next_event", "get_event"]

DEFAULT_POOL_SIZE = 16  # pool.hpp:138, :168


class event:
    """An owned CUDA event (pool.hpp:16-38; created with timing enabled, as
    ``cudaEventCreate`` does)."""

    def __init__(self):
        self.torch = torch.cuda.Event(enable_timing=True)

    def value(self) -> int:
        """The ``cudaEvent_t`` handle (0 until the event is first recorded:
        PyTorch creates the driver event lazily)."""
        return int(self.torch.cuda_event)

    def record(self, stream: "stream_view") -> None:
        """Records the event on ``stream``."""
        self.torch.record(_torch_stream(stream))

    def view(self) -> "event_view":
        return event_view(self)


class event_view:
    """A non-owning handle of an ``event`` (pool.hpp:40-63)."""

    def __init__(self, ev: event):
        if not isinstance(ev, event):
            raise TypeError("event_view wraps an event")
        self._event = ev

    @property
    def torch(self) -> torch.cuda.Event:
        return self._event.torch

    def value(self) -> int:
        return self._event.value()

    def record(self, stream: "stream_view") -> None:
        self._event.record(stream)


class stream:
    """An owned CUDA stream (pool.hpp:65-91)."""

    def __init__(self, device: Optional[Union[int, torch.device]] = None):
        self.torch = torch.cuda.Stream(device=device)

    def value(self) -> int:
        """The ``cudaStream_t`` handle."""
        return int(self.torch.cuda_stream)

    def synchronize(self) -> None:
        self.torch.synchronize()

    def wait_for_event(self, ev: Union[event, event_view]) -> None:
        """Later work on this stream waits for ``ev`` (``cudaStreamWaitEvent``)."""
        self.torch.wait_event(ev.torch)

    def as_current(self):
        """Context manager making this the current stream, so that this
        package's operators run on it."""
        return torch.cuda.stream(self.torch)

    def view(self) -> "stream_view":
        return stream_view(self)


class stream_view:
    """A non-owning handle of a stream (pool.hpp:93-120): of a ``stream``, of
    a ``torch.cuda.Stream``, or of a raw ``cudaStream_t`` given as an integer
    (0 = the legacy default stream)."""

    def __init__(self, s: Union[stream, torch.cuda.Stream, int] = 0,
                 device: Optional[Union[int, torch.device]] = None):
        if isinstance(s, stream):
            self.torch = s.torch
        elif isinstance(s, torch.cuda.Stream):
            self.torch = s
        elif isinstance(s, int):
            self.torch = (torch.cuda.default_stream(device) if s == 0
                          else torch.cuda.ExternalStream(s, device=device))
        else:
            raise TypeError("stream_view wraps a stream, a torch.cuda.Stream or a handle")

    def value(self) -> int:
        return int(self.torch.cuda_stream)

    def synchronize(self) -> None:
        self.torch.synchronize()

    def wait_for_event(self, ev: Union[event, event_view]) -> None:
        self.torch.wait_event(ev.torch)

    def as_current(self):
        return torch.cuda.stream(self.torch)


def _torch_stream(s) -> torch.cuda.Stream:
    if isinstance(s, (stream, stream_view)):
        return s.torch
    if isinstance(s, torch.cuda.Stream):
        return s
    raise TypeError("expected a stream or stream_view")


class _Pool:
    def __init__(self, make, size: int):
        size = int(size)
        if size <= 0:
            raise ValueError("pool size must be positive")
        self._items = [make() for _ in range(size)]
        self._next = itertools.count()
        self._lock = threading.Lock()

    def __len__(self) -> int:
        return len(self._items)

    def _next_item(self):
        with self._lock:  # the reference's atomic counter
            i = next(self._next)
        return self._items[i % len(self._items)]

    def _item(self, idx: int):
        return self._items[int(idx) % len(self._items)]


class stream_pool(_Pool):
    """``pool_size`` owned streams handed out as views (pool.hpp:136-164)."""

    def __init__(self, pool_size: int = DEFAULT_POOL_SIZE):
        super().__init__(stream, pool_size)

    def get_next_stream(self) -> stream_view:
        """Round-robin over the pool."""
        return stream_view(self._next_item())

    def get_stream(self, idx: int) -> stream_view:
        """Stream ``idx`` modulo the pool size."""
        return stream_view(self._item(idx))


class event_pool(_Pool):
    """``pool_size`` owned events handed out as views (pool.hpp:166-193)."""

    def __init__(self, pool_size: int = DEFAULT_POOL_SIZE):
        super().__init__(event, pool_size)

    def get_next_event(self) -> event_view:
        return event_view(self._next_item())

    def get_event(self, idx: int) -> event_view:
        return event_view(self._item(idx))


_pools = {}
_pools_lock = threading.Lock()


def _instance(kind):
    """The process-wide pool of ``kind``, created on first use on the current
    device (the reference's function-local statics, pool.hpp:195-215)."""
    with _pools_lock:
        p = _pools.get(kind)
        if p is None:
            p = _pools[kind] = stream_pool() if kind == "stream" else event_pool()
        return p


def get_next_stream() -> stream_view:
    return _instance("stream").get_next_stream()


def get_stream(idx: int) -> stream_view:
    return _instance("stream").get_stream(idx)


def get_next_event() -> event_view:
    return _instance("event").get_next_event()


def get_event(idx: int) -> event_view:
    return _instance("event").get_event(idx)
