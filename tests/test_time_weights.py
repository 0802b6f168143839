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
