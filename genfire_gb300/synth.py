"""Seeded synthetic tilt series with the shapes of the benchmark workloads.

No public dataset is involved: each workload is a volume of isotropic
Gaussian "atoms" (sampled analytically on the voxel grid), projected by the
real-space trilinear projector with the same rotation the gridding uses,
with Poisson noise at a stated mean count per pixel.  Generation uses
``numpy.random.default_rng(1000 + index)``.
"""
import numpy as np

ZYZ = ((0, 0, 1), (0, 1, 0), (0, 0, 1))
ZYX = ((0, 0, 1), (0, 1, 0), (1, 0, 0))

# name -> workload description
WORKLOADS = {
    # 64^3, 60 atoms in a sphere of radius 24, 31 single-axis tilts -75:5:75
    "tilt64": dict(index=1, D=64, atoms=60, sigma=1.5, amp=(0.5, 1.0), shape=("sphere", 24.0),
                   angles=("tilt", -75.0, 5.0, 75.0), counts=1e4, os=2.0, iters=200, vectors=ZYX, jitter=0.0),
    # 128^3, 250 atoms, radius 50, 60 random Euler triples
    "euler128": dict(index=2, D=128, atoms=250, sigma=1.2, amp=(1.0, 1.0), shape=("sphere", 50.0),
                     angles=("euler", 60, 70.0), counts=5e3, os=2.0, iters=500, vectors=ZYZ, jitter=0.0),
    # 256^3, 2000 atoms in an ellipsoid 110/110/80, 90 Euler triples, 0.3 deg jitter
    "euler256": dict(index=3, D=256, atoms=2000, sigma=1.0, amp=(0.3, 1.0), shape=("ellipsoid", 110.0, 110.0, 80.0),
                     angles=("euler", 90, 72.0), counts=None, os=2.0, iters=1000, vectors=ZYZ, jitter=0.3),
    # 512^3, 12000 atoms, radius 230, 120 Euler triples
    "euler512": dict(index=5, D=512, atoms=12000, sigma=0.9, amp=(1.0, 1.0), shape=("sphere", 230.0),
                     angles=("euler", 120, 65.0), counts=2e3, os=2.0, iters=300, vectors=ZYZ, jitter=0.0),
}


def centred(n):
    """Voxel coordinates -ceil((n-1)/2)..floor((n-1)/2) (the reference's grids)."""
    return np.arange(n) - n // 2


def support_mask(D, shape):
    """The generating sphere or ellipsoid on the centred D^3 grid (boolean, Fortran order)."""
    x = centred(D).astype(np.float64)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    if shape[0] == "sphere":
        r = shape[1]
        m = X ** 2 + Y ** 2 + Z ** 2 <= r * r
    else:
        a, b, c = shape[1:]
        m = (X / a) ** 2 + (Y / b) ** 2 + (Z / c) ** 2 <= 1.0
    return np.asfortranarray(m)


def atom_centres(rng, count, shape):
    out = []
    if shape[0] == "sphere":
        r = shape[1]
        ext = np.array([r, r, r])
    else:
        ext = np.array(shape[1:], dtype=float)
    while len(out) < count:
        c = rng.uniform(-ext, ext, size=(count, 3))
        inside = ((c / ext) ** 2).sum(axis=1) <= 1.0
        out.extend(c[inside].tolist())
    return np.array(out[:count])


def gaussian_volume(D, centres, amps, sigma, dtype=np.float32):
    """sum_a A_a exp(-|x - c_a|^2 / (2 sigma^2)) on the centred grid, window +-4 sigma."""
    vol = np.zeros((D, D, D), dtype=np.float64, order="F")
    x = centred(D).astype(np.float64)
    w = int(np.ceil(4 * sigma))
    for c, a in zip(centres, amps):
        idx = [np.arange(max(0, int(np.floor(c[k])) - w + D // 2), min(D, int(np.floor(c[k])) + w + 2 + D // 2))
               for k in range(3)]
        g = [np.exp(-(x[idx[k]] - c[k]) ** 2 / (2 * sigma * sigma)) for k in range(3)]
        vol[np.ix_(idx[0], idx[1], idx[2])] += a * g[0][:, None, None] * g[1][None, :, None] * g[2][None, None, :]
    return np.asfortranarray(vol.astype(dtype))


def angle_set(rng, spec):
    if spec[0] == "tilt":
        th = np.arange(spec[1], spec[3] + spec[2] / 2, spec[2])
        return np.stack([np.zeros_like(th), th, np.zeros_like(th)], axis=1)
    n, tmax = spec[1], spec[2]
    phi = rng.uniform(0, 360, n)
    theta = rng.uniform(-tmax, tmax, n)
    psi = rng.uniform(0, 360, n)
    return np.stack([phi, theta, psi], axis=1)


def poisson(rng, projs, counts):
    """Scale each projection to `counts` mean counts per pixel, sample, scale back."""
    out = np.empty_like(projs, dtype=np.float64)
    for p in range(projs.shape[2]):
        pj = np.clip(projs[:, :, p].astype(np.float64), 0, None)
        m = pj.mean()
        if m <= 0:
            out[:, :, p] = 0
            continue
        s = counts / m
        out[:, :, p] = rng.poisson(pj * s) / s
    return out


def make_workload(name, projector, D=None, n_proj=None, atoms=None, seed_offset=0):
    """Build a workload.

    projector(vol, angles, vectors) -> D x D x P projections.  D, n_proj and
    atoms scale a workload down (for tests); the defaults are the full
    workload.  Returns a dict with vol, support, angles (true), angles_in
    (given to the reconstructor, with jitter), projections (float64),
    vectors, os, iters.
    """
    w = dict(WORKLOADS[name])
    rng = np.random.default_rng(1000 + w["index"] + seed_offset)
    scale = 1.0
    if D is not None and D != w["D"]:
        scale = D / w["D"]
        w["D"] = D
    Dn = w["D"]
    na = atoms if atoms is not None else max(1, int(round(w["atoms"] * (scale ** 3 if scale < 1 else 1))))
    shape = w["shape"]
    if shape[0] == "sphere":
        shape = ("sphere", shape[1] * scale)
    else:
        shape = ("ellipsoid",) + tuple(s * scale for s in shape[1:])
    cents = atom_centres(rng, na, shape)
    amps = rng.uniform(w["amp"][0], w["amp"][1], na)
    vol = gaussian_volume(Dn, cents, amps, w["sigma"])
    spec = w["angles"]
    if n_proj is not None and spec[0] == "euler":
        spec = (spec[0], n_proj, spec[2])
    angles = angle_set(rng, spec)
    if n_proj is not None and spec[0] == "tilt":
        angles = angles[np.linspace(0, len(angles) - 1, n_proj).round().astype(int)]
    projs = np.asfortranarray(projector(vol, angles, w["vectors"]), dtype=np.float64)
    if w["counts"]:
        projs = np.asfortranarray(poisson(rng, projs, w["counts"]))
    angles_in = angles + (rng.normal(0, w["jitter"], angles.shape) if w["jitter"] else 0.0)
    return dict(name=name, vol=vol, support=support_mask(Dn, shape), angles=angles,
                angles_in=np.asfortranarray(angles_in), projections=projs, vectors=w["vectors"], os=w["os"],
                iters=w["iters"], D=Dn)


BATCH_SIZES = (48, 64, 96, 128, 160, 192)


def make_batch_workload(projector, count=24, seed=4, sizes=BATCH_SIZES, proj_range=(20, 80), iters=300):
    """The batched workload: `count` independent problems with object sizes
    drawn from `sizes`, 20-80 random-Euler projections each (theta in
    [-70, 70]), one Gaussian atom (sigma 1.2, amplitude 1) per 1000 voxels in a
    sphere of radius 0.4 D, Poisson noise at 1e4 counts per pixel, ZYZ axes,
    oversampling 2.  Generation uses numpy.random.default_rng(1000 + seed)."""
    rng = np.random.default_rng(1000 + seed)
    out = []
    for i in range(count):
        D = int(rng.choice(sizes))
        P = int(rng.integers(proj_range[0], proj_range[1] + 1))
        shape = ("sphere", 0.4 * D)
        na = max(1, D ** 3 // 1000)
        cents = atom_centres(rng, na, shape)
        vol = gaussian_volume(D, cents, np.ones(na), 1.2)
        angles = angle_set(rng, ("euler", P, 70.0))
        projs = np.asfortranarray(projector(vol, angles, ZYZ), dtype=np.float64)
        projs = np.asfortranarray(poisson(rng, projs, 1e4))
        out.append(dict(name="batch%d" % i, vol=vol, support=support_mask(D, shape), angles=angles,
                        angles_in=np.asfortranarray(angles), projections=projs, vectors=ZYZ, os=2.0, iters=iters,
                        D=D))
    return out
