"""Adversarial body sets shared by the oracle and GPU tests: collinear and
coplanar bodies (degenerate boxes), signed zeros and bodies exactly on the box
and split planes, a tight cluster inside a spread population (deep trees), and
two lattice clusters near the origin whose cells go past level 32."""
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


def deep(n_spread=512, seed=15):
    """Two 4x4x4 lattices (pitch 2e-12) 5e-10 apart at 1e-7 from the origin, in
    a population spread over [-1, 1]^3.  Near the origin FP32 resolves 7e-15, so
    the lattices fill cells down to level ~40, and with a softening of 1e-12
    the walk decides the MAC on cells past level 32 (their level no longer fits
    in 5 bits).  Every body pair separates within 42 levels: no key collisions."""
    rng = np.random.default_rng(seed)
    spread = rng.uniform(-1, 1, (3, n_spread)).astype(np.float32)
    g = np.arange(4, dtype=np.float64) * 2e-12
    lat = np.stack(np.meshgrid(g, g, g, indexing="ij")).reshape(3, -1) + 1e-7
    lat_b = lat.copy()
    lat_b[0] += 5e-10
    p = np.concatenate([spread, lat.astype(np.float32), lat_b.astype(np.float32)], 1)
    return _bodies(p[0], p[1], p[2], seed)


CASES = {"collinear": collinear, "coplanar": coplanar, "signed_zeros": signed_zeros, "cluster": cluster,
         "deep": deep}
# softening per case (default 0.01): the deep case needs one far below its
# cell sizes, else every cell past level ~9 passes the MAC on softening alone
EPS = {"deep": 1e-12}
