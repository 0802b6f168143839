"""Multi-step weights of the time integration (CPU): base/time/BDF.hpp and
the ramp-up of base/time/MultiStep.hpp."""
import pytest

from insilico_gb300 import workloads as W


def test_bdf_weights_ramp_up():
    """MultiStep::LHSWeights: the order ramps up over the first steps"""
    assert W.bdf_weights(2, 0) == (1.0, [1.0, -1.0])
    assert W.bdf_weights(2, 1) == (1.5, [1.5, -2.0, 0.5])
    assert W.bdf_weights(3, 1)[1] == [1.5, -2.0, 0.5]
    assert W.bdf_weights(3, 2)[1] == W.BDF_WEIGHTS[3]
    mw, w = W.inertia_weights(2, 5, 0.1)
    assert mw == pytest.approx(15.0) and w == pytest.approx([-15.0, 20.0, -5.0])


def test_adams_moulton_weights():
    """AdamsMoulton: LHS (1, -1), RHS b ramping up with the step; the
    arguments of isl_set_inertia / isl_set_force_history follow MultiStep"""
    # step 0: 0 + 2 < numRHS(3) falls back to the 2-weight rule (MultiStep.hpp:50-53)
    assert W.multistep_weights("am", 3, 0) == ([1.0, -1.0], [0.5, 0.5])
    assert W.multistep_weights("am", 3, 1) == ([1.0, -1.0], W.AM_WEIGHTS[3])
    assert W.multistep_weights("am", 2, 0) == ([1.0, -1.0], [0.5, 0.5])
    mw, w, fw = W.time_weights("am", 2, 3, 0.1)
    assert mw == pytest.approx(20.0) and w == pytest.approx([-20.0, 20.0]) and fw == pytest.approx([1.0])
    mw, w, fw = W.time_weights("bdf", 2, 3, 0.1)
    assert fw == [] and (mw, w) == W.inertia_weights(2, 3, 0.1)
