"""Seeded workload generators: deterministic, with the sizes the benchmark names."""
import numpy as np

from bonsai_gb300 import scenes as S


def test_cornell_layout():
    sd = S.cornell()
    assert sd.ntri == 12 and sd.nsph == 2 and (sd.tri_light >= 0).sum() == 2
    assert (sd.camera.width, sd.camera.height, sd.spp, sd.max_depth) == (256, 256, 16, 5)
    # walls face into the box: (p1 - p0) x (p2 - p0) points toward the origin side
    t = sd.tri.reshape(-1, 3, 3)
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    c = t.mean(axis=1)
    walls = sd.tri_light < 0
    assert (np.einsum("ij,ij->i", n[walls], -c[walls]) > 0).all()


def test_production_sizes_and_determinism():
    a = S.production(64, 36, n_ico=4, ico_level=3, n_spheres=50)
    b = S.production(64, 36, n_ico=4, ico_level=3, n_spheres=50)
    assert np.array_equal(a.tri, b.tri) and np.array_equal(a.spheres, b.spheres)
    assert a.ntri == 4 * 1280 + 2 + 8 and a.nsph == 50
    kinds = np.array([m["type"] for m in a.materials[2:]])
    assert set(np.unique(kinds)) <= {S.MATTE, S.CONDUCTOR, S.DIELECTRIC}


def test_full_production_counts():
    v, f = S.icosphere(5)
    assert len(f) == 20480
    # 64 icospheres + ground (2) + four quad lights (8)
    assert 64 * 20480 + 2 + 8 == 1_310_730


def test_ray_soup_generators():
    tri = S.random_triangles(1000, seed=1)
    t = tri.reshape(-1, 3, 3).astype(np.float64)
    e = np.linalg.norm(t[:, 1] - t[:, 0], axis=1)
    assert (e > 0.002 * 0.999).all() and (e < 0.02 * 1.001).all()
    rays = S.random_rays(5000, seed=2)
    o = rays["org"]
    on_face = np.isclose(o, 0.0) | np.isclose(o, 1.0)
    assert on_face.any(axis=1).all()
    assert np.allclose(np.linalg.norm(rays["dir"], axis=1), 1.0, atol=1e-6)
    assert np.array_equal(rays, S.random_rays(5000, seed=2))
