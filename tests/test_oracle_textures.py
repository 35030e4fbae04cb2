"""Known answers for the oracle's textures (no GPU): an image of one colour renders like the same
constant reflectance (bilinear and trilinear weights sum to one), and an image seen from so far
that the MIPMap picks its top level renders like its mean colour (Image::generate_pyramid's 2 x 2
box filter, src/io/image.rs:55-114, keeps the mean of a power-of-two image)."""
import numpy as np

import oracle as O
from bonsai_gb300 import _abi as A
from bonsai_gb300 import scenes as S


def _wall_textured(sd, tex, kd_texture=1):
    """The Cornell box with its back wall (triangles 4, 5) using `tex` through the given mapping."""
    mats = list(sd.materials) + [S.material(S.MATTE, kd=(0.0, 0.0, 0.0), kd_texture=kd_texture)]
    sd.materials = np.stack(mats)
    sd.tri_mat = sd.tri_mat.copy()
    sd.tri_mat[4:6] = len(mats) - 1
    sd.textures = [tex]
    return sd


def test_constant_image_equals_constant_reflectance():
    c = np.array([0.3, 0.55, 0.8], np.float32)
    for mapping in (A.BG_MAPPING_UV, A.BG_MAPPING_PLANAR, A.BG_MAPPING_SPHERICAL, A.BG_MAPPING_CYLINDRICAL):
        img = np.broadcast_to(c, (16, 32, 3)).astype(np.float32)
        sd = _wall_textured(S.cornell(24, 24, spp=4), S.Texture(kind=0, rgb=img, wrap=0, mapping=mapping,
                                                               uv_scale=(3.0, 2.0)))
        ref = S.cornell(24, 24, spp=4)
        mats = list(ref.materials) + [S.material(S.MATTE, kd=tuple(c))]
        ref.materials = np.stack(mats)
        ref.tri_mat = ref.tri_mat.copy()
        ref.tri_mat[4:6] = len(mats) - 1
        for mode in (A.BG_MODE_PBRT, A.BG_MODE_REF_COMPAT):
            a = O.OracleScene(sd, fixed_bvh=True).render(mode, threads=2)["rgb"]
            b = O.OracleScene(ref, fixed_bvh=True).render(mode, threads=2)["rgb"]
            np.testing.assert_allclose(a, b, rtol=2e-5, atol=1e-6)


def test_far_minified_image_filters_to_its_mean():
    rng = np.random.default_rng(4)
    img = rng.random((64, 64, 3)).astype(np.float32)
    mean = img.reshape(-1, 3).mean(0)
    # a planar mapping with a huge scale: one pixel covers thousands of texels, so the MIPMap reads
    # its 1 x 1 top level (the mean), exactly as a constant reflectance of that colour.  Depth 1:
    # only the camera ray carries differentials (later bounces read level 0, PathIntegrator
    # spawns them without differentials), so the wall's reflectance enters at the first hit only.
    sd = _wall_textured(S.cornell(24, 24, spp=16, max_depth=1), S.Texture(kind=0, rgb=img, wrap=0, mapping=A.BG_MAPPING_PLANAR,
                                                            vs=(4000.0, 0.0, 0.0), vt=(0.0, 4000.0, 0.0)))
    top = S.cornell(24, 24, spp=16, max_depth=1)
    pyr = img.copy()
    while pyr.shape[0] > 1:  # the pyramid's own f32 box filter
        pyr = ((pyr[0::2, 0::2] + pyr[0::2, 1::2] + pyr[1::2, 0::2] + pyr[1::2, 1::2]) * np.float32(0.25))
    np.testing.assert_allclose(pyr[0, 0], mean, rtol=1e-5)
    mats = list(top.materials) + [S.material(S.MATTE, kd=tuple(pyr[0, 0]))]
    top.materials = np.stack(mats)
    top.tri_mat = top.tri_mat.copy()
    top.tri_mat[4:6] = len(mats) - 1
    a = O.OracleScene(sd, fixed_bvh=True).render(A.BG_MODE_PBRT, threads=2)["rgb"]
    b = O.OracleScene(top, fixed_bvh=True).render(A.BG_MODE_PBRT, threads=2)["rgb"]
    np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-6)
