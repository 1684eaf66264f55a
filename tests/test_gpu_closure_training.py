"""The learned closure trained end to end on the GPU at a small size: a
128^3 forced stratified DNS, box filter x4 to 32^3, invariants and exact
subgrid targets on the coarse grid, Adam on the device; then what the
trained network gains a priori over dm.f's dynamic coefficient and over a
constant, and a posteriori over the coarse LES without a model."""
import numpy as np
import pytest

from sam_gb300 import closure_data as CD

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained(gpu_lib):
    params, report = CD.run(n=128, filters=(4,), n_snap=4, steps=300, batch=4096, lr=2e-3, vis=5e-3,
                            t_spinup=0.5, t_every=0.1, t_eval=0.2, out=None, log=lambda *a: None)
    return params, report


def test_training_reduces_the_loss(trained):
    _, r = trained
    assert r["samples_train"] == 3 * 32 ** 3
    assert r["loss_last"] < 0.9 * r["loss_first"]


def test_a_priori_gain(trained):
    """On the held-out snapshot the network's eddy viscosity follows the
    exact one more closely than dm.f's (a volume-averaged constant times
    |S|), its subgrid dissipation is within 20 % of the exact mean, and its
    coefficient beats the best constant in mean squared error."""
    _, r = trained
    p = r["a_priori"]
    assert p["corr_net"] > p["corr_dm"] + 0.1
    assert 0.8 < p["dissipation_net"] < 1.2
    assert p["mse_net"] < 0.95 * p["mse_mean"]


def test_a_posteriori_gain(trained):
    """Coarse LES from the filtered field, spectra against the filtered DNS
    0.2 time units later (shells k <= k_max/2): the learned closure is
    closer than no model and than dm.f."""
    _, r = trained
    e = r["a_posteriori_max_rel_err_k_le_kmax_half"]
    assert e["net"] < e["none"] and e["net"] < e["dm"]
    assert e["net"] < 0.05
