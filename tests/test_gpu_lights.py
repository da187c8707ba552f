"""Point-light rendering on the GPU against the oracle (which reproduces the
reference bit for bit on the same scene, tests/test_oracle.py): three coloured
lights of different power, one with a glTF range, at each light-distance
attenuation mode.  This exercises the light pick by the luminance CDF of the
lights' power (RenderScene.cpp:274-279, DistanceRandom.h:98-115), the coloured
intensities (PointLight.h:52-56 with main.cpp:360-362) and every branch of
computeLightAttenuation (BDPTRenderer.cpp:104-126) with and without a range
(RenderLightPoint.cpp:20-26).  Bars as in test_gpu_render.py: both sides with
their own sample variance, at most 1% of pixel-channels beyond 3 sigma and the
image mean within 4 combined standard errors."""
import os

import numpy as np
import pytest
from test_gpu_render import _render, _zstats

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("attenuation", [0, 1, 2])
def test_coloured_ranged_lights_statistically_match_oracle(gpu, oracle, scenes, attenuation):
    sc = scenes.scene_lights(40, 40, 1)
    n_cpu = 4096
    p = oracle.capi.params_for(sc, spp=n_cpu)
    p.light_distance_attenuation = attenuation
    film, sumsq, _ = oracle.OracleScene(sc).render(params=p, mode=1, threads=os.cpu_count() or 8, seed=7,
                                                   variance=True)
    ref = film[..., :3].astype(np.float64)
    var_ref = np.maximum(sumsq / n_cpu - ref ** 2, 0.0)
    n = 16384
    _, s, q, cnt, st = _render(gpu, sc, n, seed=8, lightDistanceAttenuation=attenuation)
    assert (cnt == n).all()
    mean = s / n
    var = np.maximum(q / n - mean ** 2, 0.0)
    frac3, glob = _zstats(mean, n, var, ref, n_cpu, var_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob
    assert st["light_rays"] > 0 and st["shadow_rays"] > 0

