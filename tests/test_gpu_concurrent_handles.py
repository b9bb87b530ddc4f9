"""Independent handles stepped side by side from host threads (each handle has its own stream; the
library's calls release the GIL): every simulation must equal the same simulation stepped alone,
bit for bit, and the solver statistics must be its own."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
DT = 0.01


def test_handles_in_threads_match_a_handle_alone():
    import ast_solver

    srcs = [(0.5, 0.5, 0.12, 0.06), (0.3, 0.6, 0.2, 0.08), (0.6, 0.4, 0.15, 0.05)]
    hs = [ast_solver.OctreeSmoke3(32, 3, source=src) for src in srcs]
    errs, iters = [], {}

    def run(k):
        try:
            its = []
            for _ in range(6):
                hs[k].update(DT)
                its.append(hs[k].last_solve().iterations)
            iters[k] = its
        except Exception as e:
            errs.append(e)

    th = [threading.Thread(target=run, args=(k,)) for k in range(len(hs))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs, errs
    for k, src in enumerate(srcs):
        alone = ast_solver.OctreeSmoke3(32, 3, source=src)
        its = []
        for _ in range(6):
            alone.update(DT)
            its.append(alone.last_solve().iterations)
        assert its == iters[k]
        for f in ("density_oct", "heat_oct", "mac", "tilt_vel", "p"):
            assert np.array_equal(alone.get(f), hs[k].get(f)), (k, f)
        alone.close()
        hs[k].close()
