"""CPU test of SphereScene.median_depth, the analytic median depth the full-frame
render is scored against: the distance where the optical depth of the sphere field
reaches ln 2, checked against dense numerical integration along each ray."""
import numpy as np


def _numeric_median_depth(sc, o, d, n=40001):
    d = d / np.linalg.norm(d)
    lo, hi = np.asarray(sc.aabb[0]), np.asarray(sc.aabb[1])
    with np.errstate(divide="ignore", invalid="ignore"):
        t1, t2 = (lo - o) / d, (hi - o) / d
    t0, tf = max(np.nanmax(np.minimum(t1, t2)), 0.0), np.nanmin(np.maximum(t1, t2))
    if tf <= t0:
        return np.inf
    t = np.linspace(t0, tf, n)
    p = o[None, :] + t[:, None] * d[None, :]
    cnt = (np.linalg.norm(p[:, None, :] - sc.centers[None], axis=-1) < sc.radii[None]).sum(-1)
    tau = np.concatenate([[0.0], np.cumsum(0.5 * (cnt[1:] + cnt[:-1]) * sc.density * np.diff(t))])
    k = np.nonzero(tau >= np.log(2.0))[0]
    return t[k[0]] if k.size else np.inf


def test_median_depth_matches_numeric_integration():
    from tensorf_gb300 import scene
    sc = scene.SphereScene.random(3, count=32)
    rng = np.random.default_rng(4)
    o = rng.normal(size=(60, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * 4.0
    d = -o + rng.normal(scale=0.4, size=o.shape)  # some rays miss every sphere, some miss the box
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    got = sc.median_depth(o, d)
    want = np.array([_numeric_median_depth(sc, o[i], d[i]) for i in range(len(o))])
    fin = np.isfinite(want)
    assert 0.2 < fin.mean() < 0.95  # both kinds of ray occur
    assert np.array_equal(np.isfinite(got), fin)
    np.testing.assert_allclose(got[fin], want[fin], atol=2e-4)  # the integration step is 1e-4
