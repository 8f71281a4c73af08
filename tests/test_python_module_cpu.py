"""The pybind11 module _ibisgb_py (residual / tangent / adjoint on CUDA tensors
for torch.autograd): built with the library, imports, exports its functions and
rejects host tensors before any device call (no GPU needed)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_module_exports_and_checks_its_arguments():
    from ibis_gb300 import Simulation, _ibisgb_py as py
    from tests.cases import case
    for name in ("set_conserved", "residual", "jvp", "vjp", "vjp_geometry", "jvp_geometry"):
        assert callable(getattr(py, name)), name
    g, c, st = case("ramp")
    sim = Simulation(c, g)
    U = torch.zeros(sim.num_cells, sim.n_conserved, dtype=torch.float64)
    with pytest.raises(ValueError, match="CUDA"):
        py.set_conserved(sim, U)
    with pytest.raises(ValueError, match="CUDA"):
        py.vjp(sim, U, U)
    assert np.isfinite(sim.dump("cell_geometry")).all()
