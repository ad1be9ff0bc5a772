"""Failure detection without faulting the GPU: every failure is made on the host side
(undersized pool, coincident bodies, invalid input, a wait on a flag nothing sets) and
must come back as a status code, with the sim and the context still usable."""
import ctypes as C

import numpy as np
import pytest

from helpers import gpu_sim, plummer

pytestmark = pytest.mark.gpu


def _codes():
    from nbh import _lib as L
    return L


def test_pool_exhaustion_reports_pool_error_and_sim_recovers():
    import nbh
    L = _codes()
    n = 20000
    arrs = plummer(n, seed=1)
    g = gpu_sim(pool_factor=1.0)          # 20016 nodes: 15 cells for 20000 bodies
    g.load(*arrs)
    with pytest.raises(nbh.NbhError) as ei:
        g.step()
    assert ei.value.code == L.NBH_ERR_POOL
    assert g.stats()["status"] == L.NBH_ERR_POOL
    small = plummer(1000, seed=2)         # reload: pool 16384, fits
    g.load(*small)
    g.step(2)
    assert g.stats()["status"] == 0


def test_coincident_bodies_stop_at_depth_limit():
    import nbh
    L = _codes()
    n = 4096
    x, y, z, vx, vy, vz, m = plummer(n, seed=3)
    x[7], y[7], z[7] = x[11], y[11], z[11]      # two bodies at one point never separate
    g = gpu_sim()
    g.load(x, y, z, vx, vy, vz, m)
    with pytest.raises(nbh.NbhError) as ei:
        g.step()
    assert ei.value.code == L.NBH_ERR_DEPTH
    g.load(*plummer(n, seed=4))
    g.step()
    assert g.stats()["status"] == 0


def test_invalid_inputs_rejected_at_load():
    import nbh
    L = _codes()
    n = 100
    arrs = [a.copy() for a in plummer(n, seed=5)]
    g = gpu_sim()
    with pytest.raises(nbh.NbhError) as ei:
        g.step()
    assert ei.value.code == L.NBH_ERR_STATE
    bad = [a.copy() for a in arrs]
    bad[0][3] = np.nan
    with pytest.raises(nbh.NbhError) as ei:
        g.load(*bad)
    assert ei.value.code == L.NBH_ERR_INVALID
    bad = [a.copy() for a in arrs]
    bad[6][0] = -1.0
    with pytest.raises(nbh.NbhError) as ei:
        g.load(*bad)
    assert ei.value.code == L.NBH_ERR_INVALID
    g.load(*arrs)
    g.step()


def test_bounded_wait_times_out_without_fault():
    L = _codes()
    lib = L.load()
    status = C.c_int32(0)
    L.check(lib.nbh_selftest_wait(0, 50_000_000, C.byref(status)))   # 50 ms
    assert status.value == L.NBH_ERR_TIMEOUT
    g = gpu_sim()                                                    # context still usable
    g.load(*plummer(2048, seed=6))
    g.step(3)
    assert g.stats()["status"] == 0


def test_gl_interop_mode_fills_headless_buffers():
    import torch

    import nbh
    from nbh import universe as U
    s = nbh.GPUBarnesHutNBodySimulation(nbh.Mode.GL_INTEROP, 4096, U.RandomCubicUniverseGenerator(6.0, seed=2))
    s.init(None)
    s.initGLBuffers(None, -1, -1)
    s.step()
    assert s.getNumberOfBodies() == 4096
    st = s.sim.read()
    p = s.position_buffer.cpu().numpy()
    np.testing.assert_array_equal(p[:, 0], st["x"])
    assert (p[:, 3] == 1.0).all()
    s.close()
    torch.cuda.synchronize()
