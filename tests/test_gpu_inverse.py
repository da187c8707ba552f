"""Inverse material fit through path-replay gradients on small scenes: the
roughness of the PBR materials must be recovered (its error at least halved
in 200 Adam steps), with all scenes in one group (one batch render and one
batch of adjoint jobs per step) and with the scenes one after another.  The
conductors' n, k are only weakly identifiable from RGB reflectance and are
not asserted."""
import importlib

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", ["fit", "fit_sequential"])
def test_inverse_fit_recovers_roughness(gpu, form):
    pytest.importorskip("torch")
    inv = importlib.import_module("openmaterial-validation_gb300.inverse")
    r = getattr(inv, form)(n_scenes=3, tris=10_000, res=64, spp=64, target_spp=1024, steps=200, lr=2e-2, seed=1)
    assert r.final_roughness_error < 0.5 * r.initial_roughness_error, r
