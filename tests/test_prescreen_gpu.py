"""What the trained surrogate gains over running the solver on every sweep
point: on a reduced sweep space (256-sample envelopes, 2,048 training runs,
1,024 sweep points, every one judged by the solver) the surrogate answers
far faster than the solver, its solver-judged error is well below the
no-model predictions (the input envelope delayed by the transit time, and
the mean training output), and it sorts the points of the prescreen
question mostly as the solver does."""
import pytest

pytestmark = pytest.mark.gpu


def test_surrogate_prescreen_beats_the_method_without_it(native):
    from mbsolve_gb300 import prescreen, surrogate
    sh = surrogate.Shapes(S=256, W=32, Mo=16, L=4, F=prescreen.NUM_FEATURES)
    rep, _ = prescreen.pipeline(n_train=2048, n_sweep=1024, shapes=sh,
                                epochs=20)
    assert rep["status"] == 0
    err = rep["error"]
    assert err["median"] < 0.5 * err["baseline_delayed_input_median"], err
    assert err["median"] < 0.5 * err["baseline_training_mean_median"], err
    assert rep["sweep"]["speedup"] > 20, rep["sweep"]
    assert rep["prescreen"]["accuracy"] > 0.8, rep["prescreen"]
    assert rep["train"]["loss_last"] < 0.5 * rep["train"]["loss_first"]
