"""Adversarial body sets shared by the oracle and GPU tests: collinear and
coplanar bodies (degenerate boxes), signed zeros and bodies exactly on the box
and split planes, and a tight cluster inside a spread population (deep trees)."""
import numpy as np

from nns_gb300 import ic


def _bodies(x, y, z, seed):
    n = len(x)
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((3, n)).astype(np.float32) * np.float32(0.1)
    m = np.full(n, 1.0 / n, np.float32)
    return ic.Bodies(*(np.ascontiguousarray(a, np.float32) for a in (x, y, z, v[0], v[1], v[2], m)))


def collinear(n=1500, seed=11):
    rng = np.random.default_rng(seed)
    x = np.unique(rng.uniform(-1, 1, n).astype(np.float32))
    z0 = np.zeros(len(x), np.float32)
    return _bodies(x, z0, z0.copy(), seed)


def coplanar(n=2000, seed=12):
    b = ic.star_disk(n, seed=ic.SEED0 + seed)
    return _bodies(b.x, b.y, np.zeros(len(b.x), np.float32), seed)


def signed_zeros(n=600, seed=13):
    b = ic.plummer(n, seed=ic.SEED0 + seed)
    x, y, z = b.x.copy(), b.y.copy(), b.z.copy()
    x[:40] = np.float32(-0.0)
    y[20:60] = np.float32(0.0)
    z[40:80] = np.float32(-0.0)
    # bodies on the box faces and on the first split planes
    x[100], x[101] = x.max(), x.min()
    y[102] = np.float32(0.5) * (y.max() + y.min())
    return _bodies(x, y, z, seed)


def cluster(n=1000, seed=14):
    rng = np.random.default_rng(seed)
    spread = rng.uniform(-1, 1, (3, n // 2)).astype(np.float32)
    tight = (np.float32(0.3) + rng.uniform(-1e-4, 1e-4, (3, n - n // 2))).astype(np.float32)
    p = np.concatenate([spread, tight], 1)
    return _bodies(p[0], p[1], p[2], seed)


CASES = {"collinear": collinear, "coplanar": coplanar, "signed_zeros": signed_zeros, "cluster": cluster}
