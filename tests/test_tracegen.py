"""The synthetic Manhattan generator: deterministic, on streets, inside the box."""
import numpy as np

from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator


def test_deterministic_and_chunk_independent():
    a = TraceGenerator(SEED_SCALE, 5000).steps(30)
    g = TraceGenerator(SEED_SCALE, 5000)
    b = np.concatenate([g.steps(10), g.steps(20)])
    np.testing.assert_array_equal(a, b)


def test_points_on_streets_inside_box():
    g = TraceGenerator(SEED_SCALE, 20000)
    box = g.box()
    pts = g.steps(50)
    assert (pts[..., 0] >= box[0]).all() and (pts[..., 0] <= box[2]).all()
    assert (pts[..., 1] >= box[1]).all() and (pts[..., 1] <= box[3]).all()
    # every point lies on a street line: x or y is a multiple of 100 m
    xm = (pts[..., 0] - box[0]) / (box[2] - box[0]) * 40000.0
    ym = (pts[..., 1] - box[1]) / (box[3] - box[1]) * 40000.0
    on_x = np.abs(xm - np.round(xm / 100) * 100) < 1e-3
    on_y = np.abs(ym - np.round(ym / 100) * 100) < 1e-3
    assert (on_x | on_y).all()


def test_speeds_and_stationary_fraction():
    g = TraceGenerator(SEED_SCALE, 20000)
    box = g.box()
    pts = g.steps(3)
    scale = np.array([40000.0 / (box[2] - box[0]), 40000.0 / (box[3] - box[1])])
    step = np.linalg.norm((pts[1] - pts[0]) * scale, axis=1)
    assert step.max() <= 2.0 + 1e-6
    stationary = np.mean(step == 0.0)
    assert 0.07 < stationary < 0.13


def test_hotspot_fraction():
    g = TraceGenerator(SEED_SCALE, 50000)
    pts = g.steps(1)[0]
    box = g.box()
    xm = (pts[:, 0] - box[0]) / (box[2] - box[0]) * 40000.0
    ym = (pts[:, 1] - box[1]) / (box[3] - box[1]) * 40000.0
    h, _, _ = np.histogram2d(xm, ym, bins=40, range=[[0, 40000], [0, 40000]])
    top = np.sort(h.ravel())[::-1]
    # 70% of the objects sit in 8 hotspots of sigma 500 m: a few 1 km cells hold most of them
    assert top[:64].sum() / h.sum() > 0.6
