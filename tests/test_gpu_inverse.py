"""Inverse material fit through path-replay gradients on two small scenes:
the roughness of the PBR materials must be recovered (its error at least
halved in 200 Adam steps).  The conductors' n, k are only weakly identifiable
from RGB reflectance and are not asserted."""
import importlib

import pytest

pytestmark = pytest.mark.gpu


def test_inverse_fit_recovers_roughness(gpu):
    pytest.importorskip("torch")
    inv = importlib.import_module("openmaterial-validation_gb300.inverse")
    r = inv.fit(n_scenes=2, tris=10_000, res=64, spp=64, target_spp=1024, steps=200, lr=2e-2, seed=1)
    assert r.final_roughness_error < 0.5 * r.initial_roughness_error, r
