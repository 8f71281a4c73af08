"""ibisgb_l2_norms_noalloc: residual L2 norms for callers that cannot call
cudaMalloc (device memory owned by a caching allocator such as PyTorch's, or
time loops that must not stall on cudaMalloc's device synchronization).  It
keeps its scratch in a fixed __device__ array and must give the same norms as
ibisgb_l2_norms, to rounding (the two sum in different orders), call after
call.  The cases cover one partial-sum block (8^3 = 512 cells), several blocks
whose last one is partial (24^3 = 13,824 cells: 4 blocks; 40^3 = 64,000: 16),
and a 2-D grid (4 conserved components, momentum_z norm 0).  Kept in a file
collected last."""
import ctypes as C

import numpy as np
import pytest

from ibis_gb300 import Simulation, _lib
from ibis_gb300._lib import check
from tests.cases import case

pytestmark = pytest.mark.gpu

MAX_CELLS = 16777216
CELLS_PER_BLOCK = 4096


@pytest.mark.parametrize("name,kw", [("box", {"n": 8}), ("box", {"n": 24}), ("box", {"n": 40}),
                                     ("ramp", {"ni": 96, "nj": 48})])
def test_noalloc_norms_match_the_allocating_entry_point(name, kw):
    torch = pytest.importorskip("torch")
    L = _lib.load()
    g, c, st = case(name, **kw)
    sim = Simulation(c, g)
    sim.set_primitives(*st)
    N, nc = sim.num_cells, sim.n_conserved
    if N > CELLS_PER_BLOCK:
        assert N % CELLS_PER_BLOCK != 0  # the last partial-sum block is partial
    stream = torch.cuda.current_stream()
    for _ in range(2):  # two calls in a row share (and reuse) the scratch array
        dudt = torch.empty((N, nc), dtype=torch.float64, device="cuda")
        sim.compute_dudt_into(dudt, "f64", stream=stream)
        expected = sim.L2_norms()  # the allocating entry point, on the same residual
        norms = torch.full((6,), float("nan"), dtype=torch.float64, device="cuda")
        check(L.ibisgb_l2_norms_noalloc(C.c_void_p(dudt.data_ptr()), N, nc, C.c_void_p(norms.data_ptr()),
                                        C.c_void_p(stream.cuda_stream)))
        torch.cuda.synchronize()
        got = norms.cpu().numpy()
        if nc == 4:
            assert got[4] == 0.0 and expected[4] == 0.0  # no momentum_z in 2-D
        assert np.allclose(got, expected, rtol=1e-11, atol=0), (got, expected)
        sim.take_steps(1, "f64")  # a different residual for the next call


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dudt = torch.zeros((4, 5), dtype=torch.float64, device="cuda")
    norms = torch.zeros(6, dtype=torch.float64, device="cuda")
    p, q = C.c_void_p(dudt.data_ptr()), C.c_void_p(norms.data_ptr())
    assert L.ibisgb_l2_norms_noalloc(p, MAX_CELLS + 1, 5, q, None) == -5
    assert b"num_cells" in L.ibisgb_last_error(None)
    assert L.ibisgb_l2_norms_noalloc(p, 4, 6, q, None) == -5
    assert L.ibisgb_l2_norms_noalloc(p, 0, 5, q, None) == -5
