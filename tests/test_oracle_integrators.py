"""The oracle's Whitted and direct-lighting integrators (no GPU): at max depth 1 every integrator
estimates emission + direct lighting, so their means agree with the path tracer's within Monte
Carlo error; with max depth > 1 and no specular surfaces the direct-lighting result does not
change (its recursion only follows specular lobes)."""
import numpy as np

import oracle as O
from bonsai_gb300 import _abi as A
from bonsai_gb300 import scenes as S


def test_depth_one_means_agree():
    sd = S.cornell(48, 48, spp=64, max_depth=1)
    orc = O.OracleScene(sd)
    ref = orc.render(A.BG_MODE_PBRT, spp=64)

    def mean_and_se(r):  # image mean of the sample means and its standard error
        m = r["sum"] / 64
        var = np.maximum(r["sumsq"] / 64 - m * m, 0.0) / 64
        return m.mean(), np.sqrt(var.sum()) / m.size
    m0, s0 = mean_and_se(ref)
    for kind, strategy in [(A.BG_INTEGRATOR_WHITTED, 0), (A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ALL),
                           (A.BG_INTEGRATOR_DIRECT, A.BG_LIGHT_UNIFORM_ONE)]:
        o = orc.render(A.BG_MODE_PBRT, spp=64, integrator=kind, light_strategy=strategy)
        assert o["counters"][6] == 0
        m1, s1 = mean_and_se(o)
        assert abs(m1 - m0) < 4.0 * np.hypot(s0, s1), (kind, strategy, m0, m1, s0, s1)


def test_direct_lighting_without_specular_surfaces_ignores_depth():
    sd = S.cornell(24, 24, spp=8, max_depth=1)
    sd.materials = sd.materials.copy()
    sd.materials[3] = S.material(S.MATTE, kd=(0.5, 0.5, 0.5))  # no specular lobe anywhere
    orc = O.OracleScene(sd)
    a = orc.render(A.BG_MODE_PBRT, spp=8, integrator=A.BG_INTEGRATOR_DIRECT, max_depth=1)
    b = orc.render(A.BG_MODE_PBRT, spp=8, integrator=A.BG_INTEGRATOR_DIRECT, max_depth=6)
    np.testing.assert_array_equal(a["rgb"], b["rgb"])
