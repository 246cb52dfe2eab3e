"""merc_step_static, the allocation-free entry point, against merc_step.

merc_step_static serves callers that cannot call cudaMalloc (applications
that hand the library device memory from their own pool or framework
allocator, runtimes that forbid allocation after start-up): the state stays
in the caller's device buffers and every scratch buffer of the step comes
from one fixed static device array.  This test gives it device buffers that
the test allocates itself (through torch), runs it twice in a row, and after
each call compares it with the context path (merc_step) on the same initial
state, at the tolerance of the universal-path parity tests.  The file is
named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import merc
import systems

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a = a.reshape(3, -1)
    b = b.reshape(3, -1)
    return np.max(np.abs(a - b), axis=0) / np.maximum(np.linalg.norm(b, axis=0), 1e-300)


@pytest.mark.parametrize("steps", [1, 8])
@pytest.mark.parametrize("which", ["embryo", "outer"])
def test_step_static_matches_step(which, steps):
    torch = pytest.importorskip("torch")
    # embryo disk: more than 32 massive bodies, so the kick splits its sources
    # over blocks and keeps per-chunk partial sums in the static scratch;
    # outer solar system: the per-body kernels
    sysm = systems.embryo_disk(n_embryos=254) if which == "embryo" else systems.outer_solar_system()
    n, nm = sysm.n_total, int(sysm.n_massive[0])
    params = merc.default_params(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL)
    g = merc.Integrator(params)
    g.load_systems(sysm)
    st0 = g.state()
    dev = torch.device("cuda:0")
    pos = torch.from_numpy(st0.pos.copy()).to(dev)
    vel = torch.from_numpy(st0.vel.copy()).to(dev)
    mass = torch.from_numpy(np.ascontiguousarray(sysm.mass)).to(dev)
    flags = torch.zeros(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    L = merc.lib()
    # with several steps per call the call alternates its two r_crit tables
    for call in range(2):
        g.step(steps)
        ref = g.state()
        st = L.merc_step_static(0, C.byref(params), n, nm, C.c_void_p(pos.data_ptr()), C.c_void_p(vel.data_ptr()),
                                C.c_void_p(mass.data_ptr()), C.c_void_p(flags.data_ptr()), steps, None)
        assert st == merc.MERC_OK, f"call {call}: status {st}"
        got_pos = pos.cpu().numpy()
        got_vel = vel.cpu().numpy()
        got_flags = flags.cpu().numpy().view(np.uint32)
        assert rel_err(got_pos, ref.pos).max() <= 1e-12, f"call {call}"
        assert rel_err(got_vel, ref.vel).max() <= 1e-12, f"call {call}"
        assert np.array_equal(got_flags, ref.flags), f"call {call}"
    g.close()


def test_step_static_rejects_oversize():
    torch = pytest.importorskip("torch")
    params = merc.default_params(drift=merc.DRIFT_UNIVERSAL)
    dev = torch.device("cuda:0")
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    ptr = C.c_void_p(buf.data_ptr())
    L = merc.lib()
    # ~800 bytes of scratch per body: 10 million bodies cannot fit in 16 MiB
    st = L.merc_step_static(0, C.byref(params), 10_000_000, 4, ptr, ptr, ptr, None, 1, None)
    assert st == merc.MERC_ERR_CONFIG
    # the element drift is not served by this entry point
    p2 = merc.default_params(drift=merc.DRIFT_ELEMENTS)
    assert L.merc_step_static(0, C.byref(p2), 4, 1, ptr, ptr, ptr, None, 1, None) == merc.MERC_ERR_CONFIG


def test_step_static_refuses_stream_capture():
    """The call copies small tables from its own stack and waits for its
    stream, so it must not be recorded into a graph: on a capturing stream it
    returns MERC_ERR_STATE and queues nothing."""
    torch = pytest.importorskip("torch")
    sysm = systems.outer_solar_system()
    n, nm = sysm.n_total, int(sysm.n_massive[0])
    params = merc.default_params(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL)
    dev = torch.device("cuda:0")
    buf = torch.ones(3 * n, dtype=torch.float64, device=dev)
    mass = torch.from_numpy(np.ascontiguousarray(sysm.mass)).to(dev)
    L = merc.lib()
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=s):
        buf.mul_(1.0)
        st = L.merc_step_static(0, C.byref(params), n, nm, C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()),
                                C.c_void_p(mass.data_ptr()), None, 1, C.c_void_p(s.cuda_stream))
    torch.cuda.synchronize()
    assert st == merc.MERC_ERR_STATE
