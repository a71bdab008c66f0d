"""Seeded synthetic nanoparticle models for the benchmark workloads.

Stand-ins for real structure files: spheres cut from simple-cubic, fcc and
spinel-like lattices with Gaussian jitter, FP32 coordinates grouped by
species, and the species' 11-parameter (Waasmaier & Kirfel) scattering
coefficients in the .deb column order a1..a5, b1..b5, c
(cuDebye-v15.cu:786). The coefficient rows are the published ones that the
reference ships in Matlab/Tables/atomic_scattering_factors_RIETAN.txt.

rmax follows the reference's xyz2deb converter: centre the model on its
bounding box and take Rmax = 2*ceil(1.025*max|r|) (Matlab/xyz2deb.m:198-204).

Workloads (all seeded):

* ``plain_small``   5,000 atoms, sc a=2.0 A, sigma 0.05, Al/O 40/60, B 0.5
* ``spinel_10nm``   100 A sphere of a spinel-like crystal, N ~ 118,000
* ``precision``     the spinel model with a 20,000-point q grid
* ``batch256``      256 models: sc/fcc/spinel, N log-uniform 2k..60k
* serving requests: N log-uniform 1k..200k with their own 2theta grids
"""
import math

import numpy as np

from . import Species, k_grid

# Waasmaier & Kirfel (1995) coefficients: (a1..a5, b1..b5, c).
WK = {
    "O": ((2.960427, 2.508818, 0.637853, 0.722838, 1.142756),
          (14.182259, 5.936858, 0.112726, 34.958481, 0.390240), 0.027014),
    "Al": ((4.730796, 2.313951, 1.541980, 1.117564, 3.154754),
           (3.628931, 43.051167, 0.095960, 108.932388, 1.555918), 0.139509),
    "Mg": ((4.708971, 1.194814, 1.558157, 1.170413, 3.239403),
           (4.875207, 108.506081, 0.111516, 48.292408, 1.928171), 0.126842),
    "Fe": ((12.311098, 1.876623, 3.066177, 2.070451, 6.975185),
           (5.009415, 0.014461, 18.743040, 82.767876, 0.346506), -0.304931),
    "O2-": ((3.990247, 2.300563, 0.607200, 1.907882, 1.167080),
            (16.639956, 5.636819, 0.108493, 47.299709, 0.379984), 0.025429),
    "Mg2+": ((3.062918, 4.135106, 0.853742, 1.036792, 0.852520),
             (2.015803, 4.417941, 0.065307, 9.669710, 0.187818), 0.058851),
    "Al3+": ((4.132015, 0.912049, 1.102425, 0.614876, 3.219136),
             (3.528641, 7.378344, 0.133708, 0.039065, 1.644728), 0.019397),
}


def species(name, occ=1.0, beq=0.0):
    a, b, c = WK[name]
    return Species.make(occ, beq, a, b, c)


class SynthModel:
    """A model ready for the engine: coordinates grouped by species."""

    def __init__(self, xyz, counts, names, species_params, rstep, rmax,
                 lam, tt_min, tt_max, tt_step, seed, label):
        self.xyz = xyz
        self.counts = list(counts)
        self.names = list(names)
        self.species = list(species_params)
        self.rstep, self.rmax = rstep, rmax
        self.lam, self.tt_min, self.tt_max, self.tt_step = lam, tt_min, tt_max, tt_step
        self.seed, self.label = seed, label

    @property
    def natoms(self):
        return int(sum(self.counts))

    @property
    def nbins(self):
        return int(self.rmax / self.rstep) + 2

    @property
    def pairs(self):
        """Binned pairs: sum_{a<b} n_a n_b + sum_a n_a (n_a + 1) / 2."""
        c = self.counts
        s = sum(n * (n + 1) // 2 for n in c)
        s += sum(c[i] * c[j] for i in range(len(c)) for j in range(i + 1, len(c)))
        return s

    def k_grid(self):
        return k_grid(self.lam, self.tt_min, self.tt_max, self.tt_step)

    def write_deb(self, path, device=0, block=16, grid=4096, hist=0):
        """Write a .deb file (README.md section 2 layout)."""
        with open(path, "w") as f:
            f.write("%d %d %d\n" % (device, block, grid))
            f.write("%.6f %.2f %.2f %.6g\n" % (self.lam, self.tt_min,
                                               self.tt_max, self.tt_step))
            f.write("%g %g %d\n" % (self.rmax, self.rstep, hist))
            f.write("%d\n" % len(self.counts))
            for n, name, s in zip(self.counts, self.names, self.species):
                f.write("%d %s %.4f %.4f %s %s %.6f\n" % (
                    n, name, s.occ, s.beq,
                    " ".join("%.6f" % v for v in s.a),
                    " ".join("%.6f" % v for v in s.b), s.c))
            np.savetxt(f, self.xyz, fmt="%.9g", delimiter="\t")


def xyz2deb_rmax(xyz):
    """Rmax = 2*ceil(1.025*max|r|) after centring (Matlab/xyz2deb.m:198-204)."""
    if not len(xyz):
        return 0
    x = xyz.astype(np.float64)
    c = (x.max(axis=0) + x.min(axis=0)) / 2
    d = x - c
    d *= d
    # the square root of the largest squared distance: the same value as the
    # largest square root (sqrt is correctly rounded and monotonic)
    r = math.sqrt(float((d[:, 0] + d[:, 1] + d[:, 2]).max()))
    return 2 * math.ceil(r * 1.025)


def _cube_sites(basis, a, radius):
    """All sites basis*a + cell*a within a cube covering the sphere."""
    n = int(math.ceil(radius / a)) + 1
    g = np.arange(-n, n + 1, dtype=np.float64)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 1, 3)
    return ((cells + np.asarray(basis)[None]) * a).reshape(-1, 3)


SC = [(0, 0, 0)]
FCC = [(0, 0, 0), (0, .5, .5), (.5, 0, .5), (.5, .5, 0)]
# Interstices of an fcc (cubic close-packed) anion cell.
OCT = [(.5, .5, .5), (.5, 0, 0), (0, .5, 0), (0, 0, .5)]
TET = [(x, y, z) for x in (.25, .75) for y in (.25, .75) for z in (.25, .75)]


def _closest(sites, n, rng):
    """The n sites closest to the origin (ties broken at random)."""
    d = (sites ** 2).sum(axis=1) + rng.random(len(sites)) * 1e-9
    return sites[np.argsort(d, kind="stable")[:n]]


def _finish(groups, names, params, rng, sigma, rstep, grid, seed, label):
    xyz = np.concatenate([g for g in groups]) if groups else np.zeros((0, 3))
    xyz = xyz + rng.normal(0.0, sigma, size=xyz.shape)
    xyz = xyz.astype(np.float32)
    counts = [len(g) for g in groups]
    keep = [i for i, c in enumerate(counts) if c > 0]
    off = np.cumsum([0] + counts)
    xyz = np.concatenate([xyz[off[i]:off[i + 1]] for i in keep])
    return SynthModel(xyz, [counts[i] for i in keep], [names[i] for i in keep],
                      [params[i] for i in keep], rstep, xyz2deb_rmax(xyz),
                      *grid, seed, label)


GRID_CU = (1.5406, 10.0, 130.0, 0.02)  # 6,001 points
GRID_PRECISION = (0.7107, 5.0, 150.0, 145.0 / 19999)  # 20,000 points


def plain_small(seed=0, natoms=5000):
    """sc a=2.0 A sphere of 5,000 atoms, sigma 0.05 A, Al/O assigned at
    random 40/60, B = 0.5 A^2, bin 1e-3 A, 2theta 10-130/0.02 at 1.5406 A."""
    rng = np.random.default_rng(seed)
    sites = _closest(_cube_sites(SC, 2.0, (natoms * 3 / (4 * math.pi)) ** (1 / 3) * 2.0 + 4),
                     natoms, rng)
    is_al = np.zeros(natoms, bool)
    is_al[rng.permutation(natoms)[: int(round(0.4 * natoms))]] = True
    groups = [sites[is_al], sites[~is_al]]
    params = [species("Al", 1.0, 0.5), species("O", 1.0, 0.5)]
    return _finish(groups, ["Al", "O"], params, rng, 0.05, 1e-3, GRID_CU, seed,
                   "plain_small")


def spinel(radius=50.0, a=7.9, target=118000, sigma=0.08, seed=1,
           grid=GRID_CU, rstep=1e-3, label="spinel_10nm", beq=(0.5, 0.5, 0.5)):
    """Spinel-like sphere: a cubic close-packed O2- sublattice (spinel cell
    a = 7.9 A, 32 anions per cell) cut to `radius`; cations on its
    tetrahedral (Mg2+, occupancy 0.6) and octahedral (Al3+, occupancy 0.4)
    interstices, each interstice filled at random with the probability that
    brings the total atom count to `target`."""
    rng = np.random.default_rng(seed)
    sub = a / 2  # the fcc anion sub-cell
    r2 = radius * radius
    an = _cube_sites(FCC, sub, radius)
    an = an[(an ** 2).sum(1) <= r2]
    tet = _cube_sites(TET, sub, radius)
    tet = tet[(tet ** 2).sum(1) <= r2]
    octs = _cube_sites(OCT, sub, radius)
    octs = octs[(octs ** 2).sum(1) <= r2]
    fill = min(1.0, max(0.0, (target - len(an)) / (len(tet) + len(octs))))
    tet = tet[rng.random(len(tet)) < fill]
    octs = octs[rng.random(len(octs)) < fill]
    params = [species("O2-", 1.0, beq[0]), species("Mg2+", 0.6, beq[1]),
              species("Al3+", 0.4, beq[2])]
    return _finish([an, tet, octs], ["O2-", "Mg2+", "Al3+"], params, rng,
                   sigma, rstep, grid, seed, label)


def spinel_10nm(seed=1):
    return spinel(seed=seed)


def precision(seed=1):
    """The spinel model with 20,000 q points (2theta 5-150, 0.7107 A)."""
    return spinel(seed=seed, grid=GRID_PRECISION, label="precision")


POOL = ["O", "Al", "Mg", "Fe"]


def random_model(rng, nmin, nmax, grid, label, seed):
    """One model of the batched / serving mixes: lattice uniformly sc (a=2.0),
    fcc (a=4.05) or spinel-like (a=7.9); N log-uniform in [nmin, nmax];
    1-4 species assigned at random; sigma U[0.03, 0.1]; B U[0.2, 1.5]."""
    kind = rng.integers(3)
    n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
    nsp = int(rng.integers(1, 5))
    sigma = float(rng.uniform(0.03, 0.1))
    if kind == 0:
        basis, a = SC, 2.0
    elif kind == 1:
        basis, a = FCC, 4.05
    else:
        basis, a = SPINEL_LIKE, 3.95
    dens = len(basis) / a ** 3
    radius = (3 * n / (4 * math.pi * dens)) ** (1 / 3) + 2 * a
    sites = _closest(_cube_sites(basis, a, radius), n, rng)
    sp = rng.integers(nsp, size=n)
    names = POOL[:nsp]
    params = [species(nm, 1.0, float(rng.uniform(0.2, 1.5))) for nm in names]
    groups = [sites[sp == i] for i in range(nsp)]
    return _finish(groups, names, params, rng, sigma, 1e-3, grid, seed, label)


def batch256(seed=3, nmodels=256, nmin=2000, nmax=60000):
    """256 independent models for the batched workload (cfg-0 q grid)."""
    rng = np.random.default_rng(seed)
    return [random_model(rng, nmin, nmax, GRID_CU, "batch%d" % i, seed)
            for i in range(nmodels)]


SPINEL_LIKE = FCC + [tuple(v / 2 for v in t) for t in TET[:2]] + OCT[:2]


class RequestStream:
    """Fresh serving requests at a small host cost, for arrival rates of
    hundreds per second: per lattice (sc a=2.0, fcc a=4.05, spinel-like
    a=3.95, as random_model) the sites of a sphere big enough for the
    largest request are generated and ordered by distance from the centre
    once. A request takes its N closest sites (N log-uniform), turns them by
    a random rotation, adds its own Gaussian jitter (sigma U[0.03, 0.1]),
    draws 1-4 species (each site's species uniform: a per-site random label
    drawn once, offset at random per request), B U[0.2, 1.5], and its own
    2theta grid of 2,000-20,000 points. No two requests share a geometry."""

    def __init__(self, rng, nmin=1000, nmax=200000):
        self.rng, self.nmin, self.nmax = rng, nmin, nmax
        self.sites = []
        for basis, a in ((SC, 2.0), (FCC, 4.05), (SPINEL_LIKE, 3.95)):
            dens = len(basis) / a ** 3
            radius = (3 * nmax / (4 * math.pi * dens)) ** (1 / 3) + 2 * a
            self.sites.append(_closest(_cube_sites(basis, a, radius), nmax, rng))
        # per site a uniform label in [0, 12): (label + offset) mod nsp is a
        # uniform species for nsp = 1..4 (12 is their least common multiple)
        self.labels = [rng.integers(0, 12, size=nmax).astype(np.int8)
                       for _ in self.sites]

    def next(self):
        rng = self.rng
        kind = int(rng.integers(3))
        n = int(round(math.exp(rng.uniform(math.log(self.nmin),
                                           math.log(self.nmax)))))
        nsp = int(rng.integers(1, 5))
        sigma = float(rng.uniform(0.03, 0.1))
        npts = int(rng.integers(2000, 20001))
        q, r = np.linalg.qr(rng.normal(size=(3, 3)))
        rot = q * np.sign(np.diag(r))  # a uniformly random orthogonal matrix
        # species of each site (uniform), atoms grouped by species
        lab = (self.labels[kind][:n] + np.int8(rng.integers(12))) % np.int8(nsp)
        order = np.argsort(lab, kind="stable")
        counts = np.bincount(lab, minlength=nsp).tolist()
        xyz = self.sites[kind][order] @ rot.T
        xyz += rng.normal(0.0, sigma, size=xyz.shape)
        xyz = xyz.astype(np.float32)
        keep = [i for i, c in enumerate(counts) if c > 0]
        names = [POOL[i] for i in keep]
        params = [species(nm, 1.0, float(rng.uniform(0.2, 1.5))) for nm in names]
        grid = (1.5406, 10.0, 130.0, 120.0 / (npts - 1))
        return SynthModel(xyz, [counts[i] for i in keep], names, params, 1e-3,
                          xyz2deb_rmax(xyz), *grid, None, "request")


def serving_request(rng, nmin=1000, nmax=200000):
    """One serving request: a model with its own 2theta grid of 2k-20k
    points (2theta 10-130 at 1.5406 A, step chosen for the point count)."""
    npts = int(rng.integers(2000, 20001))
    grid = (1.5406, 10.0, 130.0, 120.0 / (npts - 1))
    return random_model(rng, nmin, nmax, grid, "request", None)


def request_worker(seed, out, stop):
    """Process target (start it with the "spawn" method): RequestStream
    requests, put on the queue `out` as plain tuples (model_from_item turns
    them back into models) until the event `stop` is set."""
    import queue as queue_mod
    rs = RequestStream(np.random.default_rng(seed))
    while not stop.is_set():
        m = rs.next()
        item = (m.xyz, m.counts, m.names, [s.beq for s in m.species], m.rmax,
                m.tt_step)
        while not stop.is_set():
            try:
                out.put(item, timeout=0.1)
                break
            except queue_mod.Full:
                continue


def model_from_item(item):
    """The SynthModel of a request_worker tuple."""
    xyz, counts, names, beqs, rmax, tt_step = item
    params = [species(nm, 1.0, b) for nm, b in zip(names, beqs)]
    return SynthModel(xyz, counts, names, params, 1e-3, rmax, 1.5406, 10.0,
                      130.0, tt_step, None, "request")
