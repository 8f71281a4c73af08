"""Discrete-adjoint gradient of the ramp pressure force at the full size of the
steady-state case: the 512 x 256 Hicks-Henne ramp (15 degrees; the inflow
Mach number and the 16 bump amplitudes drawn from seed 0, as bench.py draws
them), with first-order reconstruction -- the limited second-order residual
stops falling near 2e-3, with the reference's own JFNK as well.

The gradient with respect to the Mach number and all 16 amplitudes
(ibis_gb300.adjoint, one adjoint solve) against central differences with step
1e-6 of the force between steady states re-converged at the perturbed
parameters (Newton from the base state, to an absolute residual 1e-12 of the
cold start's): every component within 1e-5 relative."""
import numpy as np
import pytest

from ibis_gb300.adjoint import gradient_check

pytestmark = pytest.mark.gpu


def test_force_gradient_matches_central_differences_at_512x256():
    out = gradient_check(512, 256, seed=0, order=1, step=1e-6)
    print("adjoint vs central differences:", out["relative_errors"])
    assert out["base_relative_residual"] <= 1e-12
    assert max(out["relative_errors"]) <= 1e-5, out
