import numpy as np
import pytest

from timfilsimmod_gb300.geometry import CONFIGS, fibonacci_sphere, icosphere, make_config, make_swimmer


@pytest.mark.parametrize("k,n", [(0, 12), (1, 42), (3, 642), (4, 2562)])
def test_icosphere_counts(k, n):
    v = icosphere(k)
    assert v.shape == (n, 3)
    np.testing.assert_allclose(np.linalg.norm(v, axis=1), 1.0, rtol=1e-14)


def test_fibonacci_unit_and_spread():
    p = fibonacci_sphere(640)
    np.testing.assert_allclose(np.linalg.norm(p, axis=1), 1.0, rtol=1e-14)
    assert abs(p.mean(axis=0)).max() < 1e-2


def test_small_config_shape_and_seeding():
    a = make_config("small", seed=1)
    b = make_config("small", seed=1)
    assert a.num_segs == 640 and a.num_blobs == 642
    np.testing.assert_array_equal(a.f_segs, b.f_segs)
    # filaments: consecutive segments 2.2 apart (straight + 1e-3 jitter)
    x = a.x_segs.reshape(32, 20, 3)
    d = np.linalg.norm(np.diff(x, axis=1), axis=2)
    np.testing.assert_allclose(d, 2.2, atol=1e-2)
    # bases sit at R + a_blob + DL/2 from the centre
    np.testing.assert_allclose(np.linalg.norm(x[:, 0], axis=1), 20 + 1 + 1.1, rtol=1e-12)


def test_beat_shapes_keep_spacing():
    s = make_swimmer(radius=30.0, subdivisions=2, nfil=50, nseg=20, shape="beat", seed=3)
    x = s.x_segs.reshape(50, 20, 3)
    np.testing.assert_allclose(np.linalg.norm(np.diff(x, axis=1), axis=2), 2.2, rtol=1e-12)


def test_config_names():
    assert set(CONFIGS) == {"small", "medium", "large"}
