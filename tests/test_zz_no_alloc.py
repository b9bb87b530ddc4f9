"""astg_mean_temperature_noalloc, the entry point whose scratch is a static device array: it gives
the same mean temperature, bit for bit, as the force stage of a handle (astg_get "ambT") on two
calls in a row, allocates no device memory, and refuses inputs larger than its scratch.

The file name sorts last so that the test also runs after every other test of the session."""
import ctypes

import numpy as np
import pytest

import ast_solver
import build_lib


@pytest.fixture(scope="module", autouse=True)
def _library():
    build_lib.build()  # no-op when the in-tree library is up to date


def _call(heat_ptr, slots, amb_ptr, errlen=256):
    err = ctypes.create_string_buffer(errlen)
    s = np.ascontiguousarray(slots, dtype=np.int64)
    st = ast_solver.lib().astg_mean_temperature_noalloc(
        heat_ptr, s.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(s), amb_ptr, None, err, errlen)
    return st, err.value.decode()


def test_sizes_beyond_the_static_scratch_are_refused():
    # the size checks come before any CUDA call, so this runs without a GPU; the pointers are
    # never dereferenced
    fake = 256
    st, msg = _call(fake, [2048 * 2048 + 1], fake)
    assert st == ast_solver.ASTG_BAD_ARG and "more than 2048 * 2048" in msg
    st, msg = _call(fake, [2048 * 2048] * 4 + [1], fake)
    assert st == ast_solver.ASTG_BAD_ARG and "8192" in msg
    st, msg = _call(fake, [1] * 7, fake)
    assert st == ast_solver.ASTG_BAD_ARG and "1..6" in msg
    st, msg = _call(fake, [0, 0], fake)
    assert st == ast_solver.ASTG_BAD_ARG and "no slots" in msg
    st, msg = _call(None, [10], fake)
    assert st == ast_solver.ASTG_BAD_ARG and "null" in msg


@pytest.mark.gpu
def test_matches_the_force_stage_on_two_calls_in_a_row():
    import torch

    dt = 0.01
    sim = ast_solver.OctreeSmoke3(16, 3)
    for _ in range(2):
        sim.update(dt)
    sim.stage(0, dt)
    sim.stage(1, dt)  # addForce: ambT of the current heat
    want = sim.get("ambT")
    heat = sim.get("heat_oct")
    slots = sim.get("level_sizes")[:, 2].astype(np.int64)
    assert slots.sum() == heat.size and np.abs(heat).max() > 0

    d_heat = torch.from_numpy(heat).cuda()
    d_amb = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ast_solver.mean_temperature_noalloc(d_heat.data_ptr(), slots, d_amb[0:].data_ptr(), stream)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    ast_solver.mean_temperature_noalloc(d_heat.data_ptr(), slots, d_amb[1:].data_ptr(), stream)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    got = d_amb.cpu().numpy()
    assert got.view(np.int64)[0] == want.view(np.int64)[0], (got[0], want[0])
    assert got.view(np.int64)[1] == want.view(np.int64)[0], (got[1], want[0])
    sim.close()


@pytest.mark.gpu
def test_host_pointer_is_refused():
    heat = np.ones(100)
    out = np.zeros(1)
    st, msg = _call(heat.ctypes.data, [100], out.ctypes.data)
    assert st == ast_solver.ASTG_BAD_ARG and "d_heat_oct" in msg
