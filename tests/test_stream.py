"""The reference's stream / event exports (stream.cu:7-36, pool.hpp):
round-robin and modulo indexing of the pools, record / wait ordering, and
this package's operators on a pool stream."""
import pytest
import torch

import curadon_gb300 as cg
from curadon_gb300 import pools as st
from curadon_gb300.phantom import ellipses_2d, fan_config

NAMES = ["event", "event_view", "event_pool", "stream", "stream_view", "stream_pool",
         "get_next_stream", "get_stream", "get_next_event", "get_event"]


def test_exports_match_the_reference():
    """The names the reference's package imports from its native module."""
    for n in NAMES:
        assert hasattr(cg, n), n
    with pytest.raises(ValueError):
        st.stream_pool(0)
    with pytest.raises(TypeError):
        st.stream_view("not a stream")


@pytest.mark.gpu
def test_pool_indexing(cuda_device):
    pool = st.stream_pool(3)
    assert len(pool) == 3
    handles = [pool.get_next_stream().value() for _ in range(6)]
    assert handles[:3] == handles[3:] and len(set(handles[:3])) == 3
    assert pool.get_stream(4).value() == pool.get_stream(1).value()  # modulo the size
    ev = st.event_pool(2)
    assert ev.get_event(5).torch is ev.get_event(1).torch
    assert cg.get_stream(17).value() == cg.get_stream(1).value()  # process-wide pool of 16


@pytest.mark.gpu
def test_record_wait_and_operators_on_a_pool_stream(cuda_device):
    g = fan_config(128, 90)
    geom = cg.FanGeometry(**g, device=cuda_device.index or 0)
    v = ellipses_2d(128, 1, device=cuda_device).contiguous()
    ref = torch.zeros(geom.sinogram_shape(), device=cuda_device)
    cg.forward(v, ref, geom)
    torch.cuda.synchronize()

    s1, s2 = cg.get_next_stream(), cg.get_next_stream()
    assert s1.value() != s2.value()
    out = torch.zeros_like(ref)
    done = cg.get_next_event()
    s1.wait_for_event(_recorded_on_current())
    with s1.as_current():
        cg.forward(v, out, geom)
    done.record(s1)
    s2.wait_for_event(done)
    copy = torch.empty_like(out)
    with s2.as_current():
        copy.copy_(out)  # ordered after the forward on s1 by the event
    s2.synchronize()
    assert torch.equal(copy, ref)
    own = st.stream()
    own.wait_for_event(done)
    own.synchronize()
    assert st.stream_view(own.value()).value() == own.value()


def _recorded_on_current():
    e = st.event()
    e.record(st.stream_view(torch.cuda.current_stream()))
    return e
