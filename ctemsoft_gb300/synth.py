"""Synthetic inputs in the reference's formats.

The reference ships no crystal, Monte-Carlo or master-pattern files, and its
producers (CTEMMC, CTEMEBSDmaster) are out of scope, so the workloads use
seeded synthetic stand-ins with the shapes, sizes and value ranges of the
named configurations:

* master pattern: FP32 on the square Lambert grid, (2npx+1)^2 x nE.  Node
  (i,j) is mapped to the sphere with the Rosca forward map
  (Lambert.f90:352-389, kvectors.f90:916-922) and given a smooth
  Kikuchi-band intensity: a background plus, for every low-index lattice
  plane of the phase, a band of half-width equal to the Bragg angle at the
  bin energy (relativistic electron wavelength), with bright edges.  Values
  are positive and O(1).  Cubic Ni (fcc) or hexagonal Ti (hcp).
* Monte-Carlo histogram accum_e: int32 (numEbins, 2nsx+1, 2nsx+1), Poisson
  counts of a smooth backscatter lobe for the tilted sample times an energy
  spectrum peaked at the beam energy, stored at the swapped Lambert pixel
  (x,y) -> (y,-x) exactly as CTEMMC.f90:494-512 bins exit directions.
* orientations: Shoemake uniform unit quaternions from numpy's
  default_rng(seed), scalar first, float32.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SPIO2 = math.sqrt(math.pi / 2.0)


def lambert_forward(X: np.ndarray, Y: np.ndarray):
    """Rosca square -> north hemisphere (double), Lambert.f90:352-389."""
    X = np.asarray(X, np.float64)
    Y = np.asarray(Y, np.float64)
    ax, ay = np.abs(X), np.abs(Y)
    yb = ax <= ay
    x = np.zeros(np.broadcast(X, Y).shape)
    y = np.zeros_like(x)
    z = np.ones_like(x)
    with np.errstate(divide="ignore", invalid="ignore"):
        q = 2.0 * Y * np.sqrt(np.pi - Y * Y) / np.pi
        qq = X * np.pi * 0.25 / Y
        xa, ya, za = q * np.sin(qq), q * np.cos(qq), 1.0 - 2.0 * Y * Y / np.pi
        q2 = 2.0 * X * np.sqrt(np.pi - X * X) / np.pi
        qq2 = Y * np.pi * 0.25 / X
        xb, yb2, zb = q2 * np.cos(qq2), q2 * np.sin(qq2), 1.0 - 2.0 * X * X / np.pi
    origin = (ax == 0) & (ay == 0)
    x = np.where(yb, xa, xb)
    y = np.where(yb, ya, yb2)
    z = np.where(yb, za, zb)
    x = np.where(origin, 0.0, x)
    y = np.where(origin, 0.0, y)
    z = np.where(origin, 1.0, z)
    return x, y, z


def electron_wavelength_nm(E_keV: float) -> float:
    V = E_keV * 1000.0
    return 1.226386 / math.sqrt(V * (1.0 + 0.97845e-6 * V))


def _unique_normals(vecs):
    out = []
    for v in vecs:
        v = np.asarray(v, np.float64)
        n = v / np.linalg.norm(v)
        if not any(abs(abs(np.dot(n, u)) - 1.0) < 1e-9 for u in out):
            out.append(n)
    return out


def plane_families(phase: str):
    """[(amplitude, d_nm, [unit normals])] of low-index planes."""
    import itertools
    fam = []
    if phase == "Ni":
        a = 0.35236
        for hkl, amp in (((1, 1, 1), 1.0), ((2, 0, 0), 0.8), ((2, 2, 0), 0.55),
                         ((3, 1, 1), 0.4)):
            vecs = set()
            for p in itertools.permutations(hkl):
                for s in itertools.product((1, -1), repeat=3):
                    vecs.add(tuple(pi * si for pi, si in zip(p, s)))
            d = a / math.sqrt(sum(h * h for h in hkl))
            fam.append((amp, d, _unique_normals(sorted(vecs))))
    elif phase == "Ti":
        a, c = 0.2951, 0.4686
        b1 = np.array([1.0, 1.0 / math.sqrt(3.0), 0.0]) / a
        b2 = np.array([0.0, 2.0 / math.sqrt(3.0), 0.0]) / a
        b3 = np.array([0.0, 0.0, 1.0 / c])
        rot60 = np.array([[0.5, -math.sqrt(3) / 2, 0], [math.sqrt(3) / 2, 0.5, 0], [0, 0, 1.0]])
        for (h, k, l), amp in (((0, 0, 2), 0.9), ((1, 0, 0), 0.6), ((1, 0, 1), 1.0),
                               ((1, 0, 2), 0.6), ((1, 1, 0), 0.5)):
            g = h * b1 + k * b2 + l * b3
            d = 1.0 / np.linalg.norm(g)
            vecs = []
            v = g.copy()
            for _ in range(6):
                vecs.append(v.copy())
                vecs.append(v * np.array([1, 1, -1.0]))
                v = rot60 @ v
            fam.append((amp, d, _unique_normals(vecs)))
    else:
        raise ValueError(f"unknown phase {phase}")
    return fam


def master_pattern(npx: int, energies, phase: str = "Ni", seed: int = 0) -> np.ndarray:
    """Synthetic master pattern shaped (nE, 2npx+1, 2npx+1) float32."""
    idx = np.arange(-npx, npx + 1, dtype=np.float64) * (SPIO2 / npx)
    X, Y = np.meshgrid(idx, idx)  # X varies along columns (Fortran x fastest)
    kx, ky, kz = lambert_forward(X, Y)
    K = np.stack([kx, ky, kz], axis=-1).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    fams = plane_families(phase)
    betas = []
    for amp, d, normals in fams:
        N = np.stack(normals)  # (m, 3)
        dots = np.abs(K @ N.T)  # (nodes, m)
        betas.append(np.arcsin(np.clip(dots, 0.0, 1.0)).astype(np.float32))
    out = np.empty((len(energies), 2 * npx + 1, 2 * npx + 1), np.float32)
    jitter = (1.0 + 1e-3 * rng.standard_normal(K.shape[0])).astype(np.float32)
    for ie, E in enumerate(energies):
        lam = electron_wavelength_nm(float(E))
        acc = np.full(K.shape[0], 1.0, np.float32)
        efac = np.float32(0.8 + 0.02 * (20.0 - float(E)))
        for (amp, d, _), beta in zip(fams, betas):
            th = np.float32(math.asin(lam / (2.0 * d)))
            u = beta / th
            prof = 1.0 / (1.0 + u ** 6) + 0.35 * np.exp(-((u - 1.0) / 0.4) ** 2) \
                - 0.12 * np.exp(-((u - 1.45) / 0.4) ** 2)
            acc += np.float32(amp) * efac * prof.sum(axis=1, dtype=np.float32)
        out[ie] = (acc * jitter).reshape(2 * npx + 1, 2 * npx + 1)
    return out


def mc_histogram(nsx: int, energies, EkeV: float, total: float = 1.0e6, seed: int = 0,
                 sig: float = 70.0) -> np.ndarray:
    """Synthetic accum_e shaped (2nsx+1, 2nsx+1, nE) int32 (Fortran (E,x,y))."""
    rng = np.random.default_rng(seed + 1000)
    i = np.arange(-nsx, nsx + 1, dtype=np.float64)
    IX, IY = np.meshgrid(i, i)  # IX along axis 1 (Fortran x), IY along axis 0
    s = SPIO2 / nsx
    # element (iy, ix) holds exit directions whose Lambert point is (-iy, ix)
    cx, cy, cz = lambert_forward(-IY * s, IX * s)
    lobe_t = np.array([math.sin(math.radians(sig - 30.0)), 0.0,
                       math.cos(math.radians(sig - 30.0))])
    d2 = (cx - lobe_t[0]) ** 2 + (cy - lobe_t[1]) ** 2 + (cz - lobe_t[2]) ** 2
    ang = np.power(np.clip(cz, 0.0, 1.0), 0.6) * (0.25 + np.exp(-d2 / (2 * 0.45 ** 2)))
    E = np.asarray(energies, np.float64)
    spec = np.exp(-(EkeV - E) / 3.5)
    lam = ang[..., None] * spec[None, None, :]
    lam *= total / lam.sum()
    return rng.poisson(lam).astype(np.int32)


def shoemake_quaternions(n: int, seed: int) -> np.ndarray:
    """Uniform random unit quaternions (scalar first), float32 (n, 4)."""
    rng = np.random.default_rng(seed)
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    t2, t3 = 2 * np.pi * u2, 2 * np.pi * u3
    q = np.stack([b * np.cos(t3), a * np.sin(t2), a * np.cos(t2), b * np.sin(t3)], axis=1)
    return q.astype(np.float32)


def misorientation_deg(a, b) -> np.ndarray:
    """Rotation angle (degrees, no crystal symmetry) between quaternion rows
    of a and b: 2 atan2(|vec(conj(a) b)|, |scalar(conj(a) b)|) in binary64,
    which keeps its accuracy near zero where arccos of the dot product
    cannot resolve angles below about 0.03 degrees from float32 inputs."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    a = a / np.linalg.norm(a, axis=1, keepdims=True)
    b = b / np.linalg.norm(b, axis=1, keepdims=True)
    s0 = (a * b).sum(axis=1)
    v = (a[:, :1] * b[:, 1:] - b[:, :1] * a[:, 1:]
         - np.cross(a[:, 1:], b[:, 1:]))
    return np.degrees(2 * np.arctan2(np.linalg.norm(v, axis=1), np.abs(s0)))


def _cached(key, make):
    """Large arrays are generated once per machine and kept as .npy files in
    $EBSD_SYNTH_CACHE (default: <tmp>/ctemsoft_gb300_synth)."""
    import hashlib
    import os
    import tempfile
    small = key[1] < 100 if isinstance(key[1], int) else False
    if small:
        return make()
    d = os.environ.get("EBSD_SYNTH_CACHE",
                       os.path.join(tempfile.gettempdir(), "ctemsoft_gb300_synth"))
    os.makedirs(d, exist_ok=True)
    path = os.path.join(d, hashlib.sha1(repr(key).encode()).hexdigest()[:20] + ".npy")
    if os.path.exists(path):
        try:
            return np.load(path)
        except Exception:
            pass
    a = make()
    tmp = path + f".{os.getpid()}.tmp.npy"
    np.save(tmp, a)
    os.replace(tmp, path)
    return a


@dataclass
class Workload:
    """One named configuration (detector, master, MC and orientations)."""
    name: str
    numsx: int
    numsy: int
    delta: float
    L: float
    thetac: float
    xpc: float
    ypc: float
    npx: int
    Ehistmin: float
    Ebinsize: float
    EkeV: float
    nEbins: int
    n_orient: int
    seed: int
    mc_nsx: int = 750
    mc_total: float = 1.0e6
    sig: float = 70.0
    phase: str = "Ni"
    binning: int = 1
    scalingmode: str = "gam"
    gammavalue: float = 0.33
    beamcurrent: float = 15.0
    dwelltime: float = 100.0
    extra: dict = field(default_factory=dict)

    @property
    def energies(self):
        return [self.Ehistmin + k * self.Ebinsize for k in range(self.nEbins)]

    def geometry(self) -> dict:
        return dict(L=self.L, thetac=self.thetac, delta=self.delta, numsx=self.numsx,
                    numsy=self.numsy, xpc=self.xpc, ypc=self.ypc, sig=self.sig)

    def master(self) -> np.ndarray:
        return _cached(("master", self.npx, tuple(self.energies), self.phase, self.seed),
                       lambda: master_pattern(self.npx, self.energies, self.phase, self.seed))

    def mc(self) -> np.ndarray:
        return _cached(("mc", self.mc_nsx, tuple(self.energies), self.EkeV, self.mc_total,
                        self.seed, self.sig),
                       lambda: mc_histogram(self.mc_nsx, self.energies, self.EkeV,
                                            self.mc_total, self.seed, self.sig))

    def quaternions(self, n: int | None = None) -> np.ndarray:
        return shoemake_quaternions(self.n_orient if n is None else n, self.seed)


# 80x60 detector, 501^2 x 11 Ni master, 100 orientations (seed 0)
C1 = Workload("plain-forward-80x60-npx250", 80, 60, 59.2, 15000.0, 10.0, 0.0, 0.0, 250, 10.0,
              1.0, 20.0, 11, 100, 0)
# 640x480 detector, 1001^2 x 11 Ni master, 10 000 orientations (seed 1)
C2 = Workload("plain-forward-640x480-npx500", 640, 480, 20.0, 15000.0, 10.0, 1.5, -3.0, 500,
              10.0, 1.0, 20.0, 11, 10000, 1)
# 480x480 detector, 1001^2 x 11 Ni master, 4096 orientations (seed 3)
C4 = Workload("adjoint-480x480-npx500", 480, 480, 20.0, 15000.0, 10.0, 0.0, 0.0, 500, 10.0, 1.0,
              20.0, 11, 4096, 3, scalingmode="not")
# 120x120 (binning 4 of 480x480), 15 bins 6-20 keV, 100 000 orientations (seed 4)
C5 = Workload("gauss-newton-480x480-bin4-npx500", 480, 480, 20.0, 15000.0, 10.0, 0.0, 0.0, 500,
              6.0, 1.0, 20.0, 15, 100000, 4, binning=4, scalingmode="lin")


C3_SIZES = [(80, 60), (160, 120), (320, 240), (640, 480), (1244, 1024)]


def c3_jobs(seed: int = 2, njobs: int = 64):
    """The batched uneven workload: njobs draws of detector size (uniform
    over C3_SIZES), binning (1, 2, 4, 8), orientation count (log-uniform in
    [1, 5000]) and phase (Ni or Ti).  Every detector spans the 12.8 mm of
    the 640x480 / 20 um camera (delta = 12800/numsx), L = 15000 um, tilt 10
    deg; gamma 0.33.  Returns dicts with keys numsx, numsy, delta, binning,
    n, phase, seed."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(njobs):
        nx, ny = C3_SIZES[int(rng.integers(0, len(C3_SIZES)))]
        b = int(rng.choice([1, 2, 4, 8]))
        n = int(np.clip(np.round(np.exp(rng.uniform(0.0, np.log(5000.0)))), 1, 5000))
        ph = "Ni" if rng.random() < 0.5 else "Ti"
        jobs.append(dict(numsx=nx, numsy=ny, delta=12800.0 / nx, binning=b, n=n, phase=ph,
                         seed=1000 + j))
    return jobs


def c3_phase(phase: str) -> Workload:
    """Master/MC workload of one C3 phase: half-width 500, 11 bins 10-20 keV."""
    return Workload(f"batched-{phase}-npx500", 640, 480, 20.0, 15000.0, 10.0, 0.0, 0.0, 500,
                    10.0, 1.0, 20.0, 11, 0, 2 if phase == "Ni" else 12, phase=phase)


def tiny(seed: int = 7, numsx: int = 24, numsy: int = 18, npx: int = 40, nE: int = 5,
         mc_nsx: int = 60, n_orient: int = 6, phase: str = "Ni") -> Workload:
    """A small workload the oracle finishes in milliseconds."""
    return Workload(f"tiny-{numsx}x{numsy}-npx{npx}", numsx, numsy, 400.0, 15000.0, 10.0, 0.7,
                    -1.3, npx, 16.0, 1.0, 20.0, nE, n_orient, seed, mc_nsx=mc_nsx,
                    mc_total=2.0e5, phase=phase)
