"""GPU tests of the DVND loop modes of one search: the device-side loop (the
default; a CUDA-graph while node, 16 iterations a pass) on the caller's
stream or on the solver's own, and host-checked graph replays of u
iterations (set_unroll(u)) give the oracle's result, with and without an
iteration cap."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,seed", [(60, 3), (400, 4)])
@pytest.mark.parametrize("cap", [None, 7, 16, 33])
def test_loop_modes_agree(mlpgpu_mod, n, seed, cap):
    import torch

    x, y = oracle.uniform_instance(n, seed)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, seed)
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=True)
    ot, ost = oracle.dvnd(t, D, max_iters=cap) if cap else oracle.dvnd(t, D)
    stream = torch.cuda.Stream()
    for mode in ("device", 16, 3, "own_stream"):
        s = mlpgpu_mod.Solver(p)
        if mode != "own_stream":
            s.set_stream(stream.cuda_stream)
        if isinstance(mode, int):
            s.set_unroll(mode)
        s.set_tour(t)
        st = s.dvnd(mlpgpu_mod.NB_ALL, cap) if cap else s.dvnd()
        assert np.array_equal(s.tour(), ot), mode
        assert st["cost"] == ost["cost"] and st["moves"] == ost["moves"], mode
        if cap is None:
            assert st["converged"] == 1 and st["sweeps"] == ost["iterations"] + 1, mode
        else:
            assert st["sweeps"] == min(cap, ost["iterations"] + 1), mode
