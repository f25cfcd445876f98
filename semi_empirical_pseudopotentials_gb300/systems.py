"""Synthetic nanocrystal inputs with the shapes of the benchmark workloads.

No public dataset is involved: every workload is a zincblende CdSe-like
sphere cut from a perfect lattice, with seeded form-factor parameters.

* Lattice: a = 6.08 Angstrom, cations on fcc sites, anions at +a/4 (1,1,1);
  atoms with |R| <= radius about a cation at the origin are kept.
* Form factor per species (pseudopotFitting/hamiltonian.c:91-94):
  v(q) = a0 (q^2 - a1) / (a2 exp(a3 q^2) + 1), with a0..a3 drawn around
  (+10, 1.5, 30, 0.3) for the cation and (-10, 1.5, 30, 0.3) for the anion,
  each scaled by 1 + 0.05 U(-1, 1) from a seeded generator.
* Real-space tables: the l = 0 sine transform of pseudopotFitting/pot.c:35-63
  with volPerAtom = a^3/8, then shifted so the last value is zero
  (filter/read.c:105-108).
* Box: half-width rint(0.5 * extent + 5) bohr per axis, grid spacing
  2 * half / n (filter/init.c:90-114); atoms centred on their mean
  (filter/read.c:16-30).

The reference's conf.par / pot<X>.par files can be written from a System so
the reference's own program reads the same inputs.
"""
from dataclasses import dataclass, field

import numpy as np

BOHR_PER_ANGSTROM = 1.0 / 0.529177210903
CATION, ANION = 0, 1  # reference type ids: Cd = 0, Se = 1 (filter/read.c:130-131)
SPECIES = {CATION: "Cd", ANION: "Se"}


def zincblende_sphere(radius_nm, a_angstrom=6.08):
    """Atoms of a zincblende sphere; returns (types[int64], xyz[natom, 3] bohr)."""
    a = a_angstrom * BOHR_PER_ANGSTROM
    rad = radius_nm * 10.0 * BOHR_PER_ANGSTROM
    n = int(np.ceil(rad / a)) + 2
    fcc = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    g = np.arange(-n, n + 1)
    cells = np.array(np.meshgrid(g, g, g, indexing="ij")).reshape(3, -1).T
    cat = ((cells[:, None, :] + fcc[None]).reshape(-1, 3)) * a
    ani = cat + a / 4.0
    keep_c = np.linalg.norm(cat, axis=1) <= rad
    keep_a = np.linalg.norm(ani, axis=1) <= rad
    xyz = np.concatenate([cat[keep_c], ani[keep_a]])
    types = np.concatenate([np.full(keep_c.sum(), CATION), np.full(keep_a.sum(), ANION)])
    return types.astype(np.int64), xyz


# The fitted zincblende CdSe form factors a0..a3 of the reference's
# pseudopotFitting/TESTS/zb_cdse (CdParams.par, SeParams.par).  With them the
# band edges of a nanocrystal converge at a few thousand Newton steps; the
# seeded a0 = +-10 set spreads the spectrum over ~80 Ha, too wide for that.
FITTED_CDSE = {CATION: np.array([0.0424846, 0.671884, 0.136082, 0.514544]),
               ANION: np.array([-0.22725, 3.69721, -2.24471, 0.676691])}


def form_factor_params(seed):
    """Seeded a0..a3 per species (see module docstring)."""
    rng = np.random.default_rng(seed)
    base = {CATION: np.array([10.0, 1.5, 30.0, 0.3]), ANION: np.array([-10.0, 1.5, 30.0, 0.3])}
    return {t: b * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, 4)) for t, b in base.items()}


@dataclass
class System:
    """Everything the filter path needs for one nanocrystal on one grid."""

    name: str
    dims: tuple            # (nx, ny, nz)
    types: np.ndarray      # [natom] reference type ids
    xyz: np.ndarray        # [natom, 3] bohr, centred
    xyz_raw: np.ndarray    # [natom, 3] bohr, as cut from the lattice
    params: dict           # type -> a0..a3
    vol_per_atom: float
    half: tuple            # box half-widths (xd, yd, zd)
    ms: int = 4
    ns: int = 8
    nc: int = 1024
    el: np.ndarray = field(default_factory=lambda: np.zeros(0))
    seed: int = 0

    @property
    def ngrid(self):
        return int(np.prod(self.dims))

    @property
    def steps(self):
        return tuple(2.0 * h / n for h, n in zip(self.half, self.dims))

    @property
    def mins(self):
        return tuple(-h for h in self.half)

    @property
    def dv(self):
        dx, dy, dz = self.steps
        return dx * dy * dz

    @property
    def natom(self):
        return len(self.types)


def _center(xyz):
    """filter/read.c:16-30: subtract the mean, summed in atom order."""
    out = np.array(xyz, dtype=np.float64, copy=True)
    for d in range(3):
        m = 0.0
        for v in out[:, d]:
            m += v
        m /= len(out)
        out[:, d] -= m
    return out


def _half(r):
    """filter/init.c:90-92: rint(0.5 * largest extent + 5)."""
    return float(np.rint(0.5 * (np.max(r) - np.min(r)) + 5.0))


def make_system(name, radius_nm, n, ms, ns, nc=1024, seed=0, el=None, elmin=None, elmax=None,
                params=None):
    """params: type -> a0..a3 (e.g. FITTED_CDSE); None draws them from `seed`."""
    types, xyz_raw = zincblende_sphere(radius_nm)
    xyz = _center(xyz_raw)
    half = tuple(_half(xyz[:, d]) for d in range(3))
    dims = (n, n, n) if np.isscalar(n) else tuple(n)
    a = 6.08 * BOHR_PER_ANGSTROM
    if el is None:
        lo = -0.40 if elmin is None else elmin
        hi = -0.10 if elmax is None else elmax
        el = lo + np.arange(ms) * ((hi - lo) / (ms - 1)) if ms > 1 else np.array([lo])
    params = form_factor_params(seed) if params is None else {t: np.asarray(v, dtype=np.float64)
                                                             for t, v in params.items()}
    return System(name=name, dims=dims, types=types, xyz=xyz, xyz_raw=xyz_raw, params=params,
                  vol_per_atom=a ** 3 / 8.0, half=half, ms=ms, ns=ns, nc=nc,
                  el=np.asarray(el, dtype=np.float64), seed=seed)


def write_reference_inputs(system, path, nthreads=8, tables=None):
    """Write input.par / conf.par / potCd.par / potSe.par for the reference.

    ``tables`` maps type -> (r[1024], v[1024]) unshifted tables (the reference
    shifts them itself on reading).  Note the box rule: the reference derives
    the box from the atoms, so the grid spacing it uses equals System.steps.
    """
    import os

    os.makedirs(path, exist_ok=True)
    with open(os.path.join(path, "input.par"), "w") as f:
        nx, ny, nz = system.dims
        f.write(f"{nx}\n{ny}\n{nz}\n{system.ms}\n{system.ns}\n{system.nc}\n")
        f.write(f"{float(system.el[0])!r}\n{float(system.el[-1])!r}\n{nthreads}\n")
    with open(os.path.join(path, "conf.par"), "w") as f:
        f.write(f"{system.natom}\n")
        for t, (x, y, z) in zip(system.types, system.xyz_raw):
            f.write(f"{SPECIES[int(t)]} {float(x)!r} {float(y)!r} {float(z)!r}\n")
    for t, (r, v) in (tables or {}).items():
        with open(os.path.join(path, f"pot{SPECIES[int(t)]}.par"), "w") as f:
            for ri, vi in zip(r, v):
                f.write(f"{float(ri)!r} {float(vi)!r}\n")


# Benchmark workloads (sizes of the benchmark configurations).
WORKLOADS = {
    "r1.2nm_64": dict(radius_nm=1.2, n=64, ms=4, ns=8, nc=1024),
    "r2.5nm_128": dict(radius_nm=2.5, n=128, ms=8, ns=64, nc=1024),
    "r4.0nm_192": dict(radius_nm=4.0, n=192, ms=8, ns=256, nc=1024),
}
