"""The FLOP basis of the roofline fraction (operation-count build of the
NODDI-Watson plugin, C1 workload: 288 measurements, 968 grid combinations,
1250 + 1250 MCMC iterations, 5 free parameters).

A change to the plugin's arithmetic changes these counts and with them the
reported TFLOP/s, so they are pinned here: 59 FLOP per signal evaluation,
41.2 FLOP of Derived_P after a one-parameter change, 2.24e8 FLOP per voxel
for MCMC and 1.74e7 for the grid search.
"""
import pytest

from cudimot_gb300 import flops


@pytest.fixture(scope="module")
def c1(built):
    return flops.watson_c1_flops_per_voxel()


def test_signal_and_derived_counts(c1):
    ops = c1["ops"]
    assert ops["signal"] == 59.0
    assert ops["signal_mufu"] == 1.0           # one exponential per measurement
    assert ops["derived_p_one_param"] == pytest.approx(41.2, abs=0.5)
    assert ops["derived_p"] == pytest.approx(169.8, abs=2.0)
    assert ops["jacobian"] > ops["signal"]


def test_per_voxel_work(c1):
    like = c1["likelihood_proposal"]
    assert like == pytest.approx(c1["ops"]["derived_p_one_param"] + 288 * (59.0 + 3.0))
    assert c1["mcmc"] == pytest.approx(2500 * 5 * like)
    assert c1["mcmc"] == pytest.approx(2.237e8, rel=5e-3)
    assert c1["gridsearch"] == pytest.approx(1.745e7, rel=5e-3)
