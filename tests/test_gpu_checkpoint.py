"""Long propagations resumed from a checkpoint on the GPU (Problem.SaveCheckpoint /
LoadCheckpoint in the layout of the reference's WavefunctionHDF serialization, written to an
.npz archive): a run interrupted half-way, saved, reloaded into a freshly built Problem and
continued ends in the same state as the uninterrupted run."""
import os

import numpy as np
import pytest

from tests.helpers import relerr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("propagator,precision", [("CayleyPropagatorGPU", "fp32"), ("CayleyPropagatorGPU", "fp64"),
                                                  ("PamPropagatorGPU", "fp64")])
def test_propagation_resumed_from_checkpoint(gpu, tmp_path, propagator, precision):
    """600 steps of the pAMP workload's model (lmax 10, 150 B-splines, 800 nm pulse; pAMP with
    its converged basis of 40) in one go, against 300 steps, a checkpoint, a new Problem
    loading it, and 300 more steps: the same propagated time and the same final state to
    rounding (the FP64 sums of some kernels are atomic, so their order can vary)."""
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import HYDROGEN_L10_PAMP, field_free_ground_state, hydrogen

    def problem():
        prob = pp.Problem(pp.LoadString(hydrogen(propagator=propagator, precision=precision,
                                                 gmres_tolerance=1e-10,
                                                 **dict(HYDROGEN_L10_PAMP, krylov_basis_size=40))))
        prob.SetupStep(skipWavefunctionSetup=True)
        return prob

    whole = problem()
    psi0, _ = field_free_ground_state(whole)
    whole.psi.SetData(psi0)
    whole.PropagatedTime = 0.0
    for _ in range(600):
        whole.AdvanceStep()

    first = problem()
    first.psi.SetData(psi0)
    first.PropagatedTime = 0.0
    for _ in range(300):
        first.AdvanceStep()
    path = os.path.join(str(tmp_path), "run.npz")
    first.SaveCheckpoint(path)
    t_saved = first.PropagatedTime
    del first

    second = problem()
    assert abs(second.LoadCheckpoint(path) - t_saved) == 0.0
    for _ in range(300):
        second.AdvanceStep()
    assert abs(second.PropagatedTime - whole.PropagatedTime) < 1e-12
    assert relerr(second.psi.numpy(), whole.psi.numpy()) < 1e-12
