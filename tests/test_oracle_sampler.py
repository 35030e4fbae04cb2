"""The StratifiedSampler (src/samplers/stratified.rs, src/base/sampling.rs:120-179) as the oracle and
the device draw it, no GPU: each stratified dimension gives every sample of a pixel's pass its own
stratum (1D: spp strata of [0, 1); 2D: an nx x ny grid), jittered inside it or at its centre;
REF_COMPAT walks the strata in sample order in every dimension (F6: `shuffle` never swaps, since
`uniform_discrete_range(0, n)` draws from Uniform(0..1)), PBRT permutes each dimension on its own;
a stratified film sample lowers the error of an image at equal spp."""
import numpy as np
import pytest

import oracle as O
from bonsai_gb300 import _abi as A
from bonsai_gb300 import scenes as S

SAMP = S.StratifiedSampler(4, 3, 4, True)


def _strata(mode, pixel, k, is2d, sampler=SAMP, pass_=0):
    n = sampler.spp
    v = np.array([O.strat_sample(sampler, mode, pixel, pass_ * n + s, k, is2d) for s in range(n)])
    if is2d:
        ix = np.floor(v[:, 0] * sampler.x_pixel_samples).astype(int)
        iy = np.floor(v[:, 1] * sampler.y_pixel_samples).astype(int)
        return v, iy * sampler.x_pixel_samples + ix
    return v, np.floor(v[:, 0] * n).astype(int)


@pytest.mark.parametrize("mode", [A.BG_MODE_PBRT, A.BG_MODE_REF_COMPAT])
@pytest.mark.parametrize("is2d", [False, True])
def test_every_sample_of_a_pass_has_its_own_stratum(mode, is2d):
    for pixel in (0, 17, 12345):
        for k in range(SAMP.sampled_dimensions):
            for pass_ in (0, 3):
                v, idx = _strata(mode, pixel, k, is2d, pass_=pass_)
                assert (v >= 0).all() and (v < 1).all()
                assert sorted(idx) == list(range(SAMP.spp))


def test_ref_compat_dimensions_share_the_stratum_order():
    """F6: sample s sits in stratum s of every dimension, 1D and 2D alike."""
    for k in range(SAMP.sampled_dimensions):
        _, i1 = _strata(A.BG_MODE_REF_COMPAT, 5, k, False)
        _, i2 = _strata(A.BG_MODE_REF_COMPAT, 5, k, True)
        assert list(i1) == list(range(SAMP.spp)) and list(i2) == list(range(SAMP.spp))


def test_pbrt_dimensions_are_permuted_independently():
    orders = {tuple(_strata(A.BG_MODE_PBRT, p, k, d)[1]) for p in (1, 2) for k in range(4) for d in (False, True)}
    assert len(orders) >= 14  # 16 (pixel, dimension) orders, essentially all distinct


def test_no_jitter_takes_the_stratum_centres():
    s = S.StratifiedSampler(4, 2, 2, False)
    v, idx = _strata(A.BG_MODE_PBRT, 9, 1, True, sampler=s)
    np.testing.assert_allclose(v[:, 0], ((idx % 4) + 0.5) / 4)
    np.testing.assert_allclose(v[:, 1], ((idx // 4) + 0.5) / 2)
    v1, idx1 = _strata(A.BG_MODE_PBRT, 9, 0, False, sampler=s)
    np.testing.assert_allclose(v1[:, 0], (idx1 + 0.5) / 8)


def test_spp_must_match_the_grid():
    sd = S.cornell(8, 8, spp=4)
    with pytest.raises(ValueError):
        O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=4, sampler=S.StratifiedSampler(3, 2, 1))


def test_dimensionless_stratified_sampler_is_the_counter_rng():
    """sampled_dimensions = 0: every call falls through to the RNG, as the independent sampler."""
    sd = S.cornell(16, 16, spp=4)
    a = O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=4)["rgb"]
    b = O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=4, sampler=S.StratifiedSampler(2, 2, 0))["rgb"]
    np.testing.assert_array_equal(a, b)


def test_stratified_film_sampling_lowers_the_error():
    """The reference's example scene at 16 spp: a 4x4 stratified sampler with 4 sampled dimensions
    against independent samples, error measured against a 1024-spp render, over 3 seeds."""
    sd = S.env_sphere(48, 48, spp=16, max_depth=3, env_w=64, env_h=32)
    ref = O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=1024, seed=99, threads=4)["rgb"]
    err = {True: 0.0, False: 0.0}
    for seed in range(3):
        for strat in (True, False):
            smp = S.StratifiedSampler(4, 4, 4, True) if strat else None
            img = O.OracleScene(sd).render(A.BG_MODE_PBRT, spp=16, seed=seed, threads=4, sampler=smp)["rgb"]
            err[strat] += float(np.mean((img - ref) ** 2))
    assert err[True] < 0.8 * err[False], err
